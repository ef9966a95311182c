// Double-float state arithmetic shared by the time step and the kernels that
// update the state in their epilogue.
#pragma once

#include <cuda_runtime.h>

namespace x3d {

// Mixed precision keeps the velocity as a double-float pair (hi, lo) of
// binary32 arrays: hi is exactly the FP32 operand the operators read, and the
// pair carries ~48 significand bits, so the state is accumulated to FP64-class
// accuracy with FP32 instructions only (GB300's FP64 pipe is 1/64 of FP32).
// (h, l) += b: two-sum of h and b, the error joined with l, renormalised.
__device__ __forceinline__ void df_add_f(float& h, float& l, float b) {
  const float s = __fadd_rn(h, b);
  const float v = __fsub_rn(s, h);
  float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, v)), __fsub_rn(b, v));
  e = __fadd_rn(e, l);
  const float hh = __fadd_rn(s, e);
  l = __fsub_rn(e, __fsub_rn(hh, s));
  h = hh;
}

}  // namespace x3d
