/* Forced include for compiling the reference's trimesh sources
 * (src/core2d/cuda/TriMesh_*.cu, filter.cc, ...) as plain host C++: under nvcc
 * those files see the CUDA headers' host min/max overloads, which g++ alone does
 * not declare.  std::min / std::max give the same results on the ints they take. */
#pragma once
#include <algorithm>
using std::max;
using std::min;
