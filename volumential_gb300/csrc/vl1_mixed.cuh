// Declarations of the mixed-precision (tensor-core) list-1 path.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "vl1.h"

namespace vl1 {

constexpr int kDigits = 5;         // signed 8-bit digits per operand
constexpr int kDigitBits = 8;
constexpr int kFixedBits = kDigits * kDigitBits;  // 40-bit fixed point

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
  int a_exp;                // 2^a_exp > max |table value|
  __nv_bfloat16 *adig;      // [key][kchunk][digit][np][kc], core-matrix K-major tiles
  int64_t adig_elems;
};

}  // namespace vl1
