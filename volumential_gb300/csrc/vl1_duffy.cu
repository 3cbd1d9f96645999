// FP64 table builder: singular box integrals by the Duffy radial scheme.
//
// Each table entry (case, source mode, target point) is
//   T = int_{[0,h]^d} G(t - y) phi_m(y) dy
// with t the case's target point, phi_m the source mode's tensor Lagrange
// basis on the Gauss-Legendre nodes of [0, h], and G a free-space kernel.
// The scheme of the reference's batched builder
// (volumential/nearfield_potential_table.py:2035-2223 for the integrand,
// :2225-2291 for the nodes): the box is split at the target point clipped
// into it into 2^d sub-boxes (one per sign vector; empty ones dropped), each
// sub-box into d! simplices (one per axis order), and each simplex is
// mapped from the unit cube by the Duffy map u_{perm(i)} = prod_{k<=i} r_k,
// whose Jacobian prod_{i<d-1} r_i^(d-1-i) cancels the singularity at the
// target; r_0 (radial) takes a tanh-sinh rule, r_1.. a Gauss-Legendre rule.
//
// GPU layout: one CTA per entry, threads striding over the quadrature nodes
// (sign vector x axis order x regular nodes x radial nodes, decoded from the
// node index; only the 1D rules are read), FP64 sums reduced per CTA.  The
// node count per entry is 2^d d! n_reg^(d-1) n_rad (3D, default orders:
// 8 x 6 x 400 x 123 = 2.4M), so the kernel is bound by the FP64 pipe.

#include <cuda_runtime.h>

#include <cstdint>

#include <algorithm>

#include "vl1_internal.cuh"

namespace vl1 {
namespace {

constexpr int kDuffyThreads = 256;
constexpr int kDuffyMaxQ = 16;

struct DuffyArgs {
  vl1_duffy_desc d;
  int n_perm, n_reg_tail, n_sub, n_chunks;
  double *part;   // [entry][chunk][re, im] partial sums
};

// axis orders in itertools.permutations order
__device__ constexpr int8_t kPerm2[2][2] = {{0, 1}, {1, 0}};
__device__ constexpr int8_t kPerm3[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2},
                                            {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};

// d/dt_a of G(dvec) (dvec = target - source) times the scaling constant,
// Laplace and Helmholtz: G'(r) d_a / r; (re, im)
template <int DIM>
__device__ __forceinline__ void green_gradient(int kind, double k, int axis, const double *dv,
                                               double &re, double &im) {
  double r2 = 0.0;
#pragma unroll
  for (int a = 0; a < DIM; ++a) r2 = fma(dv[a], dv[a], r2);
  const double da = dv[axis];
  im = 0.0;
  switch (kind) {
    case VL1_DUFFY_LAPLACE2D:   // -d_a / (2 pi r^2)
      re = -da / r2 * (0.5 / 3.141592653589793);
      break;
    case VL1_DUFFY_LAPLACE3D:   // -d_a / (4 pi r^3)
      re = -da / (r2 * sqrt(r2)) * (0.25 / 3.141592653589793);
      break;
    case VL1_DUFFY_HELMHOLTZ2D: {   // -(i/4) k H1(k r) d_a / r = (k/4)(Y1 - i J1) d_a / r
      const double r = sqrt(r2);
      const double f = 0.25 * k * da / r;
      re = f * y1(k * r);
      im = -f * j1(k * r);
      break;
    }
    default: {   // VL1_DUFFY_HELMHOLTZ3D: exp(i k r) (i k r - 1) d_a / (4 pi r^3)
      const double r = sqrt(r2);
      double sn, cs;
      sincos(k * r, &sn, &cs);
      const double f = (0.25 / 3.141592653589793) * da / (r2 * r);
      // (cs + i sn)(-1 + i k r) = (-cs - k r sn) + i (k r cs - sn)
      re = f * (-cs - k * r * sn);
      im = f * (k * r * cs - sn);
      break;
    }
  }
}

// G(dvec) times the kernel's scaling constant; (re, im)
template <int DIM>
__device__ __forceinline__ void green(int kind, double k, int power, const double *dv,
                                      double &re, double &im) {
  double r2 = 0.0;
#pragma unroll
  for (int a = 0; a < DIM; ++a) r2 = fma(dv[a], dv[a], r2);
  im = 0.0;
  switch (kind) {
    case VL1_DUFFY_LAPLACE2D:   // -log(r) / (2 pi)
      re = -0.5 * log(r2) * (0.5 / 3.141592653589793);
      break;
    case VL1_DUFFY_LAPLACE3D:   // 1 / (4 pi r)
      re = rsqrt(r2) * (0.25 / 3.141592653589793);
      break;
    case VL1_DUFFY_HELMHOLTZ2D: {   // (i/4) H0^(1)(k r) = (-Y0 + i J0) / 4
      const double kr = k * sqrt(r2);
      re = -0.25 * y0(kr);
      im = 0.25 * j0(kr);
      break;
    }
    case VL1_DUFFY_HELMHOLTZ3D: {   // exp(i k r) / (4 pi r)
      const double r = sqrt(r2);
      double s, c;
      sincos(k * r, &s, &c);
      const double f = (0.25 / 3.141592653589793) / r;
      re = c * f;
      im = s * f;
      break;
    }
    case VL1_DUFFY_CONSTANT:
      re = 1.0;
      break;
    case VL1_DUFFY_POWER:
    case VL1_DUFFY_POWER_LOG: {   // r^p (times log r): r2^(p/2), times r for odd p
      double v = 1.0;
      for (int i = 0; i < power / 2; ++i) v *= r2;
      if (power & 1) v *= sqrt(r2);
      re = kind == VL1_DUFFY_POWER ? v : v * (0.5 * log(r2));
      break;
    }
    default:   // VL1_DUFFY_PLANE_WAVE: cos(k d_0)
      re = cos(k * dv[0]);
      break;
  }
}

// One CTA per (entry, chunk) work item, or a capped grid striding over them:
// a chunk is one (sign vector, axis order) of the entry's Duffy
// sub-simplices, so an item runs for a fraction of a millisecond; the partial
// sums are added per entry in chunk order by duffy_reduce_kernel (a fixed
// order: the table is the same on every run, whatever the grid).
template <int DIM>
__global__ void __launch_bounds__(kDuffyThreads) duffy_entry_kernel(const DuffyArgs A) {
  const vl1_duffy_desc &D = A.d;
  constexpr int dim = DIM;
  const int q = D.q;
  __shared__ double s_xi[kDuffyMaxQ], s_bw[kDuffyMaxQ];
  __shared__ double s_red[2][kDuffyThreads / 32];
  if (threadIdx.x < q) {
    s_xi[threadIdx.x] = D.interp_nodes[threadIdx.x];
    s_bw[threadIdx.x] = D.interp_weights[threadIdx.x];
  }
  __syncthreads();
  // work item w = (entry, chunk); a capped grid strides over them
  const int n_chunks = A.n_chunks;
  const int64_t n_work = (int64_t)D.n_entries * n_chunks;
  for (int64_t item = blockIdx.x; item < n_work; item += gridDim.x) {
  const int e = (int)(item / n_chunks);
  const int chunk = (int)(item - (int64_t)e * n_chunks);   // isub * n_perm + iperm
  double t[3], dc[3];
  int mode[3];
  bool mode_ok = true;
#pragma unroll
  for (int a = 0; a < dim; ++a) {
    t[a] = D.target_points[(int64_t)a * D.n_entries + e];
    dc[a] = D.decomposition_targets[(int64_t)a * D.n_entries + e];
    mode[a] = D.mode_axes[(int64_t)a * D.n_entries + e];
    mode_ok = mode_ok && mode[a] >= 0 && mode[a] < q;
  }
  double *part = A.part + ((int64_t)e * n_chunks + chunk) * 2;
  if (!mode_ok) {   // an invalid entry yields NaN (the host checks its inputs)
    if (threadIdx.x == 0) {
      part[0] = __longlong_as_double(0x7FF8000000000000ll);
      part[1] = __longlong_as_double(0x7FF8000000000000ll);
    }
    continue;   // uniform across the CTA
  }
  const int iperm = chunk % A.n_perm;
  const int isub = chunk / A.n_perm;
  const int64_t n_nodes = (int64_t)A.n_reg_tail * D.n_rad;   // nodes of this chunk
  double acc_re = 0.0, acc_im = 0.0;
  for (int64_t i = threadIdx.x; i < n_nodes; i += kDuffyThreads) {
    // node index -> (regular tail node, radial node)
    const int irad = (int)(i % D.n_rad);
    int ireg = (int)(i / D.n_rad);
    // sub-box lengths along each axis (sign bit of axis a: first axis slowest)
    double len[3], sg[3];
    bool active = true;
    double len_prod = 1.0;
#pragma unroll
    for (int a = 0; a < dim; ++a) {
      sg[a] = ((isub >> (dim - 1 - a)) & 1) ? 1.0 : -1.0;
      len[a] = sg[a] < 0.0 ? dc[a] : D.extent - dc[a];
      active = active && len[a] > 0.0;
      len_prod *= len[a];
    }
    if (!active) continue;
    // unit-cube coordinates r_0 (radial), r_1.. (regular; first slowest)
    double rs[3];
    rs[0] = D.radial_nodes[irad];
    double w = D.radial_weights[irad];
#pragma unroll
    for (int a = dim - 1; a >= 1; --a) {
      const int j = ireg % D.n_reg;
      ireg /= D.n_reg;
      rs[a] = D.regular_nodes[j];
      w *= D.regular_weights[j];
    }
    // Duffy map and its Jacobian
    double cumv[3], cum = 1.0;
#pragma unroll
    for (int i2 = 0; i2 < dim; ++i2) {
      cum *= rs[i2];
      cumv[i2] = cum;
    }
    // u[perm[i2]] = cumv[i2], written as u[a] = cumv[position of a in perm]
    double u[3];
#pragma unroll
    for (int a = 0; a < dim; ++a) {
      double v = 0.0;
#pragma unroll
      for (int i2 = 0; i2 < dim; ++i2) {
        const int axis = dim == 3 ? kPerm3[iperm][i2] : kPerm2[iperm][i2];
        v = axis == a ? cumv[i2] : v;
      }
      u[a] = v;
    }
    double jac = 1.0;
#pragma unroll
    for (int i2 = 0; i2 < dim - 1; ++i2)
#pragma unroll
      for (int p = 0; p < dim - 1 - i2; ++p) jac *= rs[i2];
    // source point, displacement (target - source) and the mode's basis
    double dv[3], basis = 1.0;
#pragma unroll
    for (int a = 0; a < dim; ++a) {
      const double y = fma(sg[a] * len[a], u[a], dc[a]);
      dv[a] = t[a] - y;
      if (q > 1) {
        // first-form Lagrange polynomial: bw_m prod_{j != m} (y - x_j)
        double l = s_bw[mode[a]];
        for (int j = 0; j < q; ++j)
          if (j != mode[a]) l *= y - s_xi[j];
        basis *= l;
      }
    }
    double r2 = 0.0;
#pragma unroll
    for (int a = 0; a < dim; ++a) r2 = fma(dv[a], dv[a], r2);
    if (!(r2 > 0.0)) continue;   // a node on the singular point: zero weight
    double gre, gim;
    if (D.derivative == 0) {
      green<DIM>(D.kernel, D.k, D.power, dv, gre, gim);
    } else {
      const int axis = (D.derivative > 0 ? D.derivative : -D.derivative) - 1;
      green_gradient<DIM>(D.kernel, D.k, axis, dv, gre, gim);
      if (D.derivative < 0) {   // d/dy_a G(t - y) = -d/dt_a G
        gre = -gre;
        gim = -gim;
      }
    }
    const double f = w * jac * len_prod * basis;
    acc_re = fma(gre, f, acc_re);
    acc_im = fma(gim, f, acc_im);
  }
  // CTA reduction
  for (int o = 16; o > 0; o >>= 1) {
    acc_re += __shfl_down_sync(0xffffffffu, acc_re, o);
    acc_im += __shfl_down_sync(0xffffffffu, acc_im, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    s_red[0][warp] = acc_re;
    s_red[1][warp] = acc_im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double re = 0.0, im = 0.0;
    for (int w2 = 0; w2 < kDuffyThreads / 32; ++w2) {
      re += s_red[0][w2];
      im += s_red[1][w2];
    }
    part[0] = re;
    part[1] = im;
  }
  __syncthreads();   // s_red is reused by the next work item
  }
}

// the entries' values: their chunks' partial sums added in chunk order
__global__ void duffy_reduce_kernel(const double *part, int n_entries, int n_chunks,
                                    int complex_output, double *out) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n_entries;
       e += gridDim.x * blockDim.x) {
    double re = 0.0, im = 0.0;
    for (int c = 0; c < n_chunks; ++c) {
      re += part[((int64_t)e * n_chunks + c) * 2];
      im += part[((int64_t)e * n_chunks + c) * 2 + 1];
    }
    if (complex_output) {
      out[2 * (int64_t)e] = re;
      out[2 * (int64_t)e + 1] = im;
    } else {
      out[e] = re;
    }
  }
}

}  // namespace
}  // namespace vl1

using namespace vl1;

extern "C" int32_t vl1_duffy_table(const vl1_duffy_desc *desc, double *result, void *stream) {
  if (!desc || !result) {
    set_error("vl1_duffy_table: null descriptor or result");
    return VL1_E_ARG;
  }
  const vl1_duffy_desc &D = *desc;
  if (D.dim < 2 || D.dim > 3 || D.q < 1 || D.q > kDuffyMaxQ || D.n_entries < 0 ||
      D.n_reg < 1 || D.n_rad < 1 || !(D.extent > 0.0) || D.kernel < 0 ||
      D.kernel > VL1_DUFFY_POWER_LOG) {
    set_error("vl1_duffy_table: dim %d, q %d, entries %d, rules %d/%d, extent %g or kernel %d "
              "out of range", D.dim, D.q, D.n_entries, D.n_reg, D.n_rad, D.extent, D.kernel);
    return VL1_E_ARG;
  }
  if (D.derivative != 0 &&
      (D.derivative > D.dim || D.derivative < -D.dim || D.kernel > VL1_DUFFY_HELMHOLTZ3D)) {
    set_error("vl1_duffy_table: derivative %d of kernel %d not supported (Laplace and "
              "Helmholtz first derivatives along an axis)", D.derivative, D.kernel);
    return VL1_E_ARG;
  }
  if ((D.kernel == VL1_DUFFY_POWER && (D.power < 0 || D.power > 64)) ||
      (D.kernel == VL1_DUFFY_POWER_LOG && (D.power < 1 || D.power > 64))) {
    set_error("vl1_duffy_table: power %d out of range for kernel %d", D.power, D.kernel);
    return VL1_E_ARG;
  }
  if (D.n_entries == 0) return VL1_OK;
  if (!D.target_points || !D.decomposition_targets || !D.mode_axes || !D.regular_nodes ||
      !D.regular_weights || !D.radial_nodes || !D.radial_weights || !D.interp_nodes ||
      !D.interp_weights) {
    set_error("vl1_duffy_table: null array in the descriptor");
    return VL1_E_ARG;
  }
  DuffyArgs A;
  A.d = D;
  A.n_perm = D.dim == 3 ? 6 : 2;
  A.n_reg_tail = D.dim == 3 ? D.n_reg * D.n_reg : D.n_reg;
  A.n_sub = 1 << D.dim;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // partial sums per (entry, chunk): stream-ordered scratch, so that a build
  // never waits for work on other streams
  const int n_chunks = A.n_sub * A.n_perm;
  void *scratch = nullptr;
  cudaError_t e = lib_malloc_async(&scratch, sizeof(double) * 2 * (size_t)D.n_entries * n_chunks, s);
  if (e != cudaSuccess) return cuda_fail(e, "allocation of the Duffy partial sums");
  A.part = static_cast<double *>(scratch);
  A.n_chunks = n_chunks;
  // one CTA per (entry, chunk), or at most max_ctas CTAs striding over them
  // (a build that must leave most SMs to other work)
  const int64_t n_work = (int64_t)D.n_entries * n_chunks;
  const int64_t cap = D.max_ctas > 0 ? D.max_ctas : n_work;
  const dim3 grid((unsigned)std::min<int64_t>(std::min(n_work, cap), 0x7FFFFFFF));
  if (D.dim == 3)
    duffy_entry_kernel<3><<<grid, kDuffyThreads, 0, s>>>(A);
  else
    duffy_entry_kernel<2><<<grid, kDuffyThreads, 0, s>>>(A);
  e = cudaGetLastError();
  if (e == cudaSuccess) {
    const int blocks = (int)std::min<int64_t>(((int64_t)D.n_entries + 255) / 256, 4096);
    duffy_reduce_kernel<<<blocks, 256, 0, s>>>(A.part, D.n_entries, n_chunks, D.complex_output,
                                               result);
    e = cudaGetLastError();
  }
  cudaFreeAsync(scratch, s);
  return e == cudaSuccess ? VL1_OK : cuda_fail(e, "duffy_entry_kernel launch");
}
