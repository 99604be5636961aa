// Project-written subset of GLM (see GLM/glm.hpp).  TEST INFRASTRUCTURE ONLY.
#pragma once
#include "../glm.hpp"
namespace glm {
template <class T> T pi() { return T(3.14159265358979323846264338327950288); }
}
