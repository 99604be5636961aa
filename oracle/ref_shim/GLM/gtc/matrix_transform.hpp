// Project-written subset of GLM (see GLM/glm.hpp): rotate() lives there.
// TEST INFRASTRUCTURE ONLY.
#pragma once
#include "../glm.hpp"
