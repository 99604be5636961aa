// Stand-in for CellarWorkbench's Grid3D (not vendored by the reference): a
// dense 3D array with the accessors TextureSampler uses (construction with an
// optional fill value, get / set / operator[] by cell index).
#pragma once

#include <vector>

#include <GLM/glm.hpp>

namespace cellar {

template <class T>
class Grid3D
{
public:
    Grid3D(int w, int h, int d, const T& fill = T()) : _w(w), _h(h), _d(d), _v((size_t)w * h * d, fill) {}
    typename std::vector<T>::reference get(int i, int j, int k) { return _v[index(i, j, k)]; }
    typename std::vector<T>::const_reference get(int i, int j, int k) const { return _v[index(i, j, k)]; }
    void set(int i, int j, int k, const T& v) { _v[index(i, j, k)] = v; }
    typename std::vector<T>::reference operator[](const glm::ivec3& p) { return get(p.x, p.y, p.z); }
    typename std::vector<T>::const_reference operator[](const glm::ivec3& p) const { return get(p.x, p.y, p.z); }

private:
    size_t index(int i, int j, int k) const { return ((size_t)k * _h + j) * _w + i; }
    int _w, _h, _d;
    std::vector<T> _v;
};

}  // namespace cellar
