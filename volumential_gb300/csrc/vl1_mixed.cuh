// Declarations of the mixed-precision (tensor-core) list-1 path.
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#include "vl1.h"

namespace vl1 {

constexpr int kDigits = 5;         // 8-bit digits per operand (held exactly in FP16)
constexpr int kDigitBits = 8;
// Both operands are 39-bit fixed-point magnitudes in balanced base-256
// digits (|digit| <= 128) carrying the value's sign: a diagonal sum of digit
// products over K <= 128 source points is at most 2^22 in magnitude for
// i + j <= 3, where one FP32 addition recovers its integer bits.
constexpr int kFixedBits = kDigits * kDigitBits - 1;   // table: 39 bits + sign
constexpr int kXFixedBits = kDigits * kDigitBits - 1;  // densities: 39 bits + sign

// Operand geometry of one plan.
struct MixedGeom {
  int kp;    // source points padded (multiple of kc)
  int kc;    // K chunk (<= 64): one exact tensor-core accumulation
  int n_kc;  // kp / kc
  int np;    // output columns padded: q^d (real) or 2 q^d (complex), multiple of nch
  int nch;   // output columns per CTA: 16, 32 or 64
};

struct MixedPlan {
  MixedGeom geom;
  double table_absmax;      // largest |table value| (real and imaginary parts)
  int adig_alloc;           // index of adig in the plan's allocations
  int a_exp;                // 2^a_exp > max |table value|
  __half *adig;             // [key][kchunk][digit][np][kc] FP16 digits, swizzled K-major tiles
  int64_t adig_elems;
};

}  // namespace vl1
