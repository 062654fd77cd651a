/* Stand-in for cusp/array1d.h (cusp is not available offline), used ONLY to
 * compile the reference's src/core3d/cuda/meshFIM3dEikonal.cu for pinning its
 * host set-up (gettetmem).  The reference uses cusp::array1d as a thrust vector
 * (meshFIM3dEikonal.h:14-16), so the stand-in is thrust's host/device vectors. */
#pragma once
#include <thrust/device_vector.h>
#include <thrust/host_vector.h>
namespace cusp {
struct host_memory {};
struct device_memory {};
template <class T, class M> struct array1d_sel;
template <class T> struct array1d_sel<T, host_memory> { using type = thrust::host_vector<T>; };
template <class T> struct array1d_sel<T, device_memory> { using type = thrust::device_vector<T>; };
template <class T, class M> using array1d = typename array1d_sel<T, M>::type;
}  // namespace cusp
