// Instantiations of the line kernels for one operator kind (K_DPV); split
// out so the kernel variants compile in parallel.
#include "x3d_line_fast.cuh"

namespace x3d {
namespace lk {
template <>
int line_dispatch<K_DPV>(const LineArgs<double>& a, bool xl, int lmax, dim3 grid, size_t smem, cudaStream_t st) {
  return dispatch_xl<double, K_DPV>(a, xl, lmax, grid, smem, st);
}
template <>
int line_dispatch<K_DPV>(const LineArgs<float>& a, bool xl, int lmax, dim3 grid, size_t smem, cudaStream_t st) {
  return dispatch_xl<float, K_DPV>(a, xl, lmax, grid, smem, st);
}
template <>
int fast_dispatch<K_DPV>(const FastArgs<float>& a, bool xl, int L, dim3 grid, size_t smem, cudaStream_t st) {
  return fast_dispatch_xl<float, K_DPV>(a, xl, L, grid, smem, st);
}
}  // namespace lk
}  // namespace x3d
