// Fused D3Q27 entropic LB step: pull streaming with boundary links, moments,
// product-form equilibrium, entropic alpha, beta-relaxation.  One thread per node.
//
// Replaces, for the D3Q27 lattice, the per-level chain
// streaming -> calculate_flow_variables -> collision of
// looping/timestepping/loop.f95:104-139.  The reference has no D3Q27 collision
// (its equilibria exist only for D3Q19/D3Q39, amr/modules/amr_processes.f95:1501-1747);
// the physics here is the product-form ELBM (Karlin, Boesch, Chikatamarla 2014)
// with the reference's D3Q27 ordering and boundary-link semantics.
//
// Pull form of the reference's push streaming (streaming.f95:266-481): the
// population j that arrives at node x comes from the link that leaves x along
// -c_j.  Interior links read fout_j(x - c_j); every boundary rule of the
// reference writes its result at the source node (fi(x, opp(i)) = ...), so it
// becomes a read of a word-described source in the previous step's buffer.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "../../include/elbm_gb300.h"
#include "kernels.cuh"
#include "lattice.cuh"
#include "dfloat.cuh"
#include "mlp.cuh"
#include "mlp_tc.cuh"

namespace elbm {

// Learned-alpha network weights for inference: every thread reads the same
// weight at the same time, so constant memory feeds them to the FMAs directly.
__constant__ float c_mlp[kMlpParams];

void upload_alpha_mlp(const float* w_host, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(c_mlp, w_host, sizeof(float) * kMlpParams, 0, cudaMemcpyHostToDevice, s);
}

namespace {

constexpr int Q = Q27;

__device__ __forceinline__ int64_t nbr_offset(int j, int nx, int64_t nxy) {
  // flat offset of x + c_j
  return (int64_t)cx27(j) + (int64_t)cy27(j) * nx + (int64_t)cz27(j) * nxy;
}

template <typename T>
__device__ __forceinline__ T load_src(const T* __restrict__ src, int64_t plane, int pop, int64_t node) {
  return __ldg(src + (int64_t)pop * plane + node);
}

// Row and plane strides of the box holding node n.
__device__ __forceinline__ void box_strides(const Step27Args& a, int64_t n, int& nx, int64_t& nxy) {
  if (a.nbox <= 1) {
    nx = a.nx;
    nxy = (int64_t)a.nx * a.ny;
  } else {
    const int4 bd = __ldg(a.boxdim + __ldg(a.chunk_box + (n >> 5)));
    nx = bd.x;
    nxy = (int64_t)bd.x * bd.y;
  }
}

// Population j of boundary node n (record b) as its link word w says.
template <typename T>
__device__ __forceinline__ T pull_link(const Step27Args& a, const T* __restrict__ src, int64_t n, int32_t b, int j,
                                       uint16_t w, int nx, int64_t nxy) {
  const T* __restrict__ eq = static_cast<const T*>(a.eq);
  const int kind = lw_kind(w);
  if (kind == LK_PULL) {
    const int off = lw_off(w);
    const int64_t s = n + (int64_t)(off % 3 - 1) + (int64_t)((off / 3) % 3 - 1) * nx + (int64_t)(off / 9 - 1) * nxy;
    return load_src(src, a.plane, lw_pop(w), s);
  }
  if (kind == LK_XBOX) return load_src(src, a.plane, lw_pop(w), (int64_t)__ldg(a.xsrc + (int64_t)b * Q + j));
  if (kind == LK_EQ) return eq[lw_pop(w) * Q + j];
  if (kind == LK_IBB) {
    // linear interpolated bounce-back (Bouzidi, Firdaouss, Lallemand 2001) in pull form:
    // q < 1/2: f_j = 2q f*_i(x) + (1 - 2q) f*_i(x + c_j); q >= 1/2: f_j = f*_i(x)/(2q) + (1 - 1/(2q)) f*_j(x)
    // (the same combination holds for deviations: w_i = w_j)
    const int i = lw_pop(w), off = lw_off(w);
    const T q = __ldg(static_cast<const T*>(a.qfrac) + (int64_t)b * Q + j);
    const T fi = load_src(src, a.plane, i, n);
    if (q < (T)0.5 && off != 13) {
      const int64_t s2 = (off == kOffXbox) ? (int64_t)__ldg(a.xsrc + (int64_t)b * Q + j)
                                           : n + (int64_t)(off % 3 - 1) + (int64_t)((off / 3) % 3 - 1) * nx +
                                                 (int64_t)(off / 9 - 1) * nxy;
      return (T)2 * q * fi + ((T)1 - (T)2 * q) * load_src(src, a.plane, i, s2);
    }
    if (q >= (T)0.5) return fi / ((T)2 * q) + ((T)1 - (T)1 / ((T)2 * q)) * load_src(src, a.plane, j, n);
    return fi;
  }
  return load_src(src, a.plane, j, n);
}

// Gather the 27 streamed populations of node n (pull), bulk or boundary.
// rec: the node's boundary record when the caller knows it (-1: look it up).
template <typename T>
__device__ __forceinline__ void gather(const Step27Args& a, const T* __restrict__ src, int64_t n, uint8_t t,
                                       T (&f)[Q], int32_t rec = -1) {
  int nx;
  int64_t nxy;
  box_strides(a, n, nx, nxy);
  if (t == NT_BULK) {
#pragma unroll
    for (int j = 0; j < Q; ++j) f[j] = load_src(src, a.plane, j, n - nbr_offset(j, nx, nxy));
  } else {
    const int32_t b = rec >= 0 ? rec : __ldg(a.bidx + n);
    const uint16_t* __restrict__ wp = a.words + (int64_t)b * Q;
#pragma unroll
    for (int j = 0; j < Q; ++j) f[j] = pull_link(a, src, n, b, j, __ldg(wp + j), nx, nxy);
  }
}

// The pulls of boundary record b (node n) from its resolved sources: one
// 32-bit word per population (record-minor), below 2^31 the element of the
// source buffer, with the top bit set an entry of the equilibrium tables,
// all ones a link that needs its word (interpolated bounce-back).
template <typename T>
__device__ __forceinline__ void gather_resolved(const Step27Args& a, const T* __restrict__ src, int64_t n, int32_t b,
                                                T (&f)[Q]) {
  const T* __restrict__ eq = static_cast<const T*>(a.eq);
  uint32_t k[Q];
#pragma unroll
  for (int j = 0; j < Q; ++j) k[j] = __ldg(a.rsrc + (int64_t)j * a.nbnd + b);
#pragma unroll
  for (int j = 0; j < Q; ++j) {
    if (k[j] < 0x80000000u) {
      f[j] = __ldg(src + k[j]);
    } else if (k[j] != 0xffffffffu) {
      f[j] = eq[k[j] & 0x7fffffffu];
    } else {
      int nx;
      int64_t nxy;
      box_strides(a, n, nx, nxy);
      f[j] = pull_link(a, src, n, b, j, __ldg(a.words + (int64_t)b * Q + j), nx, nxy);
    }
  }
}

// The 27 pulls of a bulk node (all interior links of its own box).
// One base pointer per thread; with one box per level the 27 offsets
// j plane - (c_j . strides) are the same for every thread of the launch.
template <typename T>
__device__ __forceinline__ void gather_bulk(const Step27Args& a, const T* __restrict__ src, int64_t n, T (&f)[Q]) {
  int nx;
  int64_t nxy;
  box_strides(a, n, nx, nxy);
  const T* __restrict__ p = src + n;
#pragma unroll
  for (int j = 0; j < Q; ++j) f[j] = __ldg(p + ((int64_t)j * a.plane - nbr_offset(j, nx, nxy)));
}

// The same pulls at offsets computed once per launch (one-box levels).
template <typename T>
__device__ __forceinline__ void gather_bulk_off(const Step27Args& a, const T* __restrict__ src, int64_t n,
                                                T (&f)[Q]) {
  const T* __restrict__ p = src + n;
#pragma unroll
  for (int j = 0; j < Q; ++j) f[j] = __ldg(p + a.pull_off[j]);
}

// Streaming (evict-first) stores: the new populations are not read again before
// the next step, and a level larger than L2 would only push out the lines that
// neighbouring warps' pulls still share (+0.9% on the 512x256x256 level).
template <typename T>
__device__ __forceinline__ void store_dst(T* __restrict__ dst, int64_t plane, int64_t n, const T (&f)[Q]) {
  T* __restrict__ p = dst + n;
#pragma unroll
  for (int j = 0; j < Q; ++j) __stcs(p + (int64_t)j * plane, f[j]);
}

__device__ __forceinline__ void warp_stats(DevStats* st, bool active, unsigned iters, bool exact, bool fb,
                                           unsigned flags, double dH) {
  st += (blockIdx.x & (kStatSlots - 1)) * kStatStride;
  const unsigned mask = __activemask();
  const unsigned nover = __popc(__ballot_sync(mask, (flags & 0x8u) != 0));
  const unsigned nact = __popc(__ballot_sync(mask, active));
  const unsigned nexact = __popc(__ballot_sync(mask, exact));
  const unsigned nfb = __popc(__ballot_sync(mask, fb));
  const unsigned sit = __reduce_add_sync(mask, iters);
  const unsigned fl = __reduce_or_sync(mask, flags);
  // maximum of the 64-bit pattern of a non-negative double: high word first, then low word
  const unsigned long long bits = (unsigned long long)__double_as_longlong(dH);
  const unsigned hi = __reduce_max_sync(mask, (unsigned)(bits >> 32));
  const unsigned lo = __reduce_max_sync(mask, ((unsigned)(bits >> 32) == hi) ? (unsigned)bits : 0u);
  const int leader = __ffs(mask) - 1;
  if ((int)(threadIdx.x & 31) == leader) {
    if (nact) atomicAdd(&st->node_updates, (unsigned long long)nact);
    if (sit) atomicAdd(&st->newton_iters, (unsigned long long)sit);
    if (nexact) atomicAdd(&st->exact_nodes, (unsigned long long)nexact);
    if (nfb) atomicAdd(&st->fallbacks, (unsigned long long)nfb);
    if (fl) atomicOr(&st->status, fl);
    if (nover) atomicAdd(&st->dh_over, (unsigned long long)nover);
    const unsigned long long m = ((unsigned long long)hi << 32) | lo;
    if (m) atomicMax(&st->max_dH_bits, m);
  }
}

// Per-thread statistics of the nodes a persistent thread updates, added to the
// level's counters once at the end (a warp's atomics per node would all hit
// the same few addresses).
// Counts are packed two to a word (a thread of a persistent launch updates at
// most 2^31 / 65,536 < 2^16 nodes of a level).
struct StatAcc {
  unsigned nodes_exact = 0;  // nodes (low half), exact-path nodes (high half)
  unsigned fb_over = 0;      // Newton fallbacks (low half), |dH| above tolerance (high half)
  unsigned iters = 0, flags = 0;
  double dH = 0.0;
};

__device__ __forceinline__ void flush_stats(DevStats* st, const StatAcc& s) {
  st += (blockIdx.x & (kStatSlots - 1)) * kStatStride;
  const unsigned m = 0xffffffffu;
  const unsigned nodes = __reduce_add_sync(m, s.nodes_exact & 0xffffu), iters = __reduce_add_sync(m, s.iters);
  const unsigned exact = __reduce_add_sync(m, s.nodes_exact >> 16), fb = __reduce_add_sync(m, s.fb_over & 0xffffu);
  const unsigned over = __reduce_add_sync(m, s.fb_over >> 16), fl = __reduce_or_sync(m, s.flags);
  const unsigned long long bits = (unsigned long long)__double_as_longlong(s.dH);
  const unsigned hi = __reduce_max_sync(m, (unsigned)(bits >> 32));
  const unsigned lo = __reduce_max_sync(m, ((unsigned)(bits >> 32) == hi) ? (unsigned)bits : 0u);
  if ((threadIdx.x & 31) == 0) {
    if (nodes) atomicAdd(&st->node_updates, (unsigned long long)nodes);
    if (iters) atomicAdd(&st->newton_iters, (unsigned long long)iters);
    if (exact) atomicAdd(&st->exact_nodes, (unsigned long long)exact);
    if (fb) atomicAdd(&st->fallbacks, (unsigned long long)fb);
    if (fl) atomicOr(&st->status, fl);
    if (over) atomicAdd(&st->dh_over, (unsigned long long)over);
    const unsigned long long mx = ((unsigned long long)hi << 32) | lo;
    if (mx) atomicMax(&st->max_dH_bits, mx);
  }
}

// ---------------------------------------------------------------------------
// Entropy difference in the conservation-consistent form (see the oracle):
//   G(alpha) = H(f + alpha Delta) - H(f) = sum_i f_i psi(y_i, alpha),
//   y_i = Delta_i / f_i,  psi(y, a) = phi(a y) - a y ln(1 + y),
//   phi(x) = (1 + x) ln(1 + x) - x,
// exact when Delta conserves mass and momentum (it does analytically; the
// dropped terms a*sum D (1 + ln feq/w) are pure rounding residuals, which the
// direct form would amplify by 1/|Delta|^2 into alpha).
// ---------------------------------------------------------------------------

__device__ __forceinline__ double phi64(double x) {
  if (fabs(x) < 1e-2) {
    double p = 1.0 / 132.0;
#pragma unroll
    for (int n = 11; n >= 2; --n) p = fma(p, -x, 1.0 / (n * (n - 1.0)));
    return x * x * p;
  }
  return fma(1.0 + x, log1p(x), -x);
}

// ---------------------------------------------------------------------------
// FP64 path: populations f_i in FP64, Newton from alpha = 2, tolerance on the
// step; same algorithm and stopping rules as the CPU oracle.
// ---------------------------------------------------------------------------

__device__ double entropy_diff64(const double (&f)[Q], const double (&d)[Q], const double (&L1)[Q], double alpha) {
  double g = 0.0;
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    const double y = d[i] / f[i];
    g += f[i] * (phi64(alpha * y) - alpha * y * L1[i]);
  }
  return g;
}

__device__ double alpha_newton64(const double (&f)[Q], const double (&d)[Q], double tol, double tol_dH, int max_it,
                                 unsigned& iters, bool& fallback) {
  double L1[Q];
  double s2 = 0.0, amax = INFINITY;
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    L1[i] = log1p(d[i] / f[i]);
    s2 += d[i] * d[i] / f[i];
    if (d[i] < 0.0) amax = fmin(amax, -f[i] / d[i]);
  }
  iters = 0;
  fallback = false;
  if (s2 < 1e-30) return 2.0;
  double alpha = (2.0 < amax) ? 2.0 : 0.5 * (1.0 + amax);
  bool ok = false;
  for (int it = 0; it < max_it; ++it) {
    double g = 0.0, gp = 0.0;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      const double y = d[i] / f[i];
      g += f[i] * (phi64(alpha * y) - alpha * y * L1[i]);
      gp += d[i] * (log1p(alpha * y) - L1[i]);
    }
    iters = it + 1;
    if (!(gp > 0.0)) break;
    const double step = g / gp;
    double next = alpha - step;
    // a Newton step that leaves the bracket (1, amax) is replaced by halving the way to its end
    const bool clipped = !(next > 1.0) || !(next < amax);
    if (!(next > 1.0)) next = 0.5 * (alpha + 1.0);
    else if (!(next < amax)) next = 0.5 * (alpha + amax);
    alpha = next;
    if (!clipped && fabs(step) <= tol) {
      ok = true;
      break;
    }
  }
  if (!ok) {
    if ((int)iters >= max_it && fabs(entropy_diff64(f, d, L1, alpha)) <= tol_dH) return alpha;
    fallback = true;
    return (2.0 < amax) ? 2.0 : 0.5 * (1.0 + amax);
  }
  return alpha;
}

__global__ void __launch_bounds__(128) d3q27_fp64_kernel(const Step27Args a) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.N) return;
  const uint8_t t = __ldg(a.ntype + n);
  if (t == NT_SKIP) return;
  const double* __restrict__ src = static_cast<const double*>(a.src);
  double* __restrict__ dst = static_cast<double*>(a.dst);
  double f[Q];
  gather(a, src, n, t, f);

  double rho = 0.0, jx = 0.0, jy = 0.0, jz = 0.0;
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    rho += f[i];
    jx += cx27(i) * f[i];
    jy += cy27(i) * f[i];
    jz += cz27(i) * f[i];
  }
  const double u[3] = {jx / rho, jy / rho, jz / rho};
  // entropic equilibrium: prod_a w1 psi(u_a) zeta(u_a)^c_ia
  double g[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double sq = sqrt(1.0 + 3.0 * u[k] * u[k]);
    const double psi = 2.0 - sq;
    const double zeta = (2.0 * u[k] + sq) / (1.0 - u[k]);
    g[k][1] = (2.0 / 3.0) * psi;
    g[k][2] = (1.0 / 6.0) * psi * zeta;
    g[k][0] = (1.0 / 6.0) * psi / zeta;
  }
  double d[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) d[i] = rho * g[0][cx27(i) + 1] * g[1][cy27(i) + 1] * g[2][cz27(i) + 1] - f[i];

  double alpha = 2.0;
  unsigned iters = 0;
  bool fb = false;
  double dH = 0.0;
  if (a.alpha_mode != 0) {
    alpha = alpha_newton64(f, d, a.tol_alpha, a.tol_dH, a.max_newton, iters, fb);
    if (a.check_dH) {
      double L1[Q];
#pragma unroll
      for (int i = 0; i < Q; ++i) L1[i] = log1p(d[i] / f[i]);
      dH = fabs(entropy_diff64(f, d, L1, alpha));
    }
  }
  unsigned flags = 0;
  if (!isfinite(rho) || !isfinite(u[0]) || !isfinite(u[1]) || !isfinite(u[2])) flags |= 0x1u;
  if (fb) flags |= 0x2u;
  if (a.check_dH && dH > a.tol_dH) flags |= 0x8u;
  const double ab = alpha * a.beta;
  bool neg = false;
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    f[i] = f[i] + ab * d[i];
    neg |= f[i] < 0.0;
  }
  if (neg) flags |= 0x4u;
  if (neg && a.neg_list) {
#pragma unroll
    for (int i = 0; i < Q; ++i)
      if (f[i] < 0.0) {
        const unsigned long long slot = atomicAdd(a.neg_count, 1ull);
        if ((long long)slot < a.neg_cap) a.neg_list[slot] = (unsigned long long)n * Q + i;
      }
  }
  store_dst(dst, a.plane, n, f);
  if (a.alpha_out) a.alpha_out[n] = (float)alpha;
  warp_stats(a.stats, true, iters, false, fb, flags, dH);
}

// ---------------------------------------------------------------------------
// FP32 path: deviations d_i = f_i - w_i stored in FP32; collision in FP32.
//
// Entropic alpha without cancellation.  With y_i = Delta_i / f_i and the power
// sums S_n = sum_i f_i y_i^n, the entropy difference divided by alpha is
//   g(alpha) = G(alpha)/alpha = sum_n [b_n + a_n alpha^(n-1)] S_n,
//   a_n = (-1)^n / (n(n-1)),  b_n = -(-1)^n / (n-1),
// (the Taylor series of psi(y, alpha)/alpha in y).  Around alpha = 2 the S_2
// terms cancel analytically:
//   g(2 + delta) = sum_n [c0_n + a_n P_{n-1}(delta)] S_n,
//   c0_n = a_n 2^(n-1) + b_n  (c0_2 = 0),  P_m = (2 + delta)^m - 2^m,
// with P_m built by P_m = (2 + delta) P_{m-1} + delta 2^(m-1), so g is
// evaluated from small quantities only and Newton runs on delta in FP32.
// Populations with |y| > kYSmall, where the series converges slowly, are
// summed individually (rare: strongly non-equilibrium nodes), in FP32 with a
// cancellation-free form, and in float pairs where FP32 cannot resolve the
// entropy difference to the tolerance.
// ---------------------------------------------------------------------------

constexpr float kYSmall = 0.1f;
// One series order for every node: at |y| <= 0.1 the truncation leaves
// |g| ~ f (2|y|)^13 / 338 <= 1e-12, and a single instantiation keeps the
// kernel's code small enough for the instruction caches.
constexpr int kSeriesK = 12;

__host__ __device__ constexpr double pow2i(int e) {
  double r = 1.0;
  for (int i = 0; i < e; ++i) r *= 2.0;
  return r;
}
__host__ __device__ constexpr double a_n(int n) { return ((n & 1) ? -1.0 : 1.0) / (n * (n - 1.0)); }
__host__ __device__ constexpr double b_n(int n) { return -((n & 1) ? -1.0 : 1.0) / (n - 1.0); }
__host__ __device__ constexpr double c0_n(int n) { return a_n(n) * pow2i(n - 1) + b_n(n); }

struct AlphaOut {
  float delta;     // alpha = 2 + delta + delta_lo
  float delta_lo;  // low part, non-zero after a float-pair solve
  unsigned iters;
  bool large;      // some population took the individual (non-series) route
  bool fallback;
};

// Series of 2 atanh: with s = x/(2+x), ln(1+x) = 2 s A(s^2),
// A(z) = 1 + z/3 + z^2/5 + ..., and B(z) = (A(z) - 1)/z = 1/3 + z/5 + ...;
// eight terms reach FP32 rounding for |s| <= 1/3 (-1/2 <= x <= 1), 24 terms
// for |s| <= 0.6 (x >= -0.75); s^2 <= 0.36 beyond that is not reached by the
// populations of a node inside its positivity bracket at alpha near 2.
__device__ __forceinline__ void atanh_series(float s2, float& A, float& B) {
  float a, b;
  if (s2 <= 1.0f / 9.0f) {
    a = 1.0f / 17.0f;
    b = 1.0f / 19.0f;
#pragma unroll
    for (int k = 7; k >= 0; --k) {
      a = fmaf(a, s2, 1.0f / (2 * k + 1));
      b = fmaf(b, s2, 1.0f / (2 * k + 3));
    }
  } else {
    a = 1.0f / 49.0f;
    b = 1.0f / 51.0f;
#pragma unroll 4
    for (int k = 23; k >= 0; --k) {
      a = fmaf(a, s2, 1.0f / (2 * k + 1));
      b = fmaf(b, s2, 1.0f / (2 * k + 3));
    }
  }
  A = a;
  B = b;
}

// psi(y, alpha) = phi(alpha y) - alpha y ln(1 + y) for one strongly
// non-equilibrium population, without the cancellation of its O(y^2) terms:
// with x = alpha y, s_x = x/(2+x), s_y = y/(2+y), delta = alpha - 2,
//   psi = alpha y^2 (2 delta - x) / ((2+x)(2+y))
//         + 2 (1+x) s_x^3 B(s_x^2) - 2 alpha y s_y^3 B(s_y^2)
// (the O(y^2) parts of phi(x) = x^2/(2+x) + 2(1+x) s_x^3 B and of
// alpha y ln(1+y) = 2 alpha y s_y (1 + s_y^2 B) are combined exactly).
// dlog = ln(1 + alpha y) - ln(1 + y), for the derivative.
__device__ __forceinline__ void psi_large(float y, float alpha, float delta, float& psi, float& dlog, float& mag) {
  const float x = alpha * y;
  const float sx = __fdividef(x, 2.0f + x), sy = __fdividef(y, 2.0f + y);
  float Ax, Bx, Ay, By;
  atanh_series(sx * sx, Ax, Bx);
  atanh_series(sy * sy, Ay, By);
  const float t1 = __fdividef(alpha * y * y * fmaf(2.0f, delta, -x), (2.0f + x) * (2.0f + y));
  const float t2 = 2.0f * (1.0f + x) * sx * sx * sx * Bx;
  const float t3 = 2.0f * alpha * y * sy * sy * sy * By;
  psi = t1 + t2 - t3;
  mag = fabsf(t1) + fabsf(t2) + fabsf(t3);
  dlog = 2.0f * fmaf(sx, Ax, -sy * Ay);
}

// FP32 sum over the flagged populations (|y| > kYSmall):
// G_L(alpha) = sum f psi(y, alpha), G_L'(alpha) = sum f y [ln(1 + alpha y) - ln(1 + y)],
// and GLabs = sum f (|t1| + |t2| + |t3|), the scale of the rounding error of G_L.
struct LargePop {
  float f, y, ylo;  // y + ylo = Delta / f to float-pair accuracy
};
__device__ __forceinline__ void large_terms(const LargePop* lp, int nl, float alpha, float delta, float& GL,
                                            float& GLp, float& GLabs) {
  GL = 0.f;
  GLp = 0.f;
  GLabs = 0.f;
  for (int k = 0; k < nl; ++k) {
    float ps, dl, mg;
    psi_large(lp[k].y, alpha, delta, ps, dl, mg);
    GL = fmaf(lp[k].f, ps, GL);
    GLp = fmaf(lp[k].f * lp[k].y, dl, GLp);
    GLabs = fmaf(lp[k].f, mg, GLabs);
  }
}

// Float-pair sum over a list of populations:
// G = sum f [(1 + x) ln(1 + x) - x - x ln(1 + y)], x = alpha y (the entropy
// difference H(f + alpha Delta) - H(f) of those populations, conservation-
// consistent form), and its derivative G' = sum f y [ln(1 + x) - ln(1 + y)]
// in FP32 (Newton needs it to a few digits only).
__device__ __noinline__ void df_terms(const LargePop* lp, int nl, df alpha, df& G, float& Gp) {
  G = df_make(0.f);
  Gp = 0.f;
  for (int k = 0; k < nl; ++k) {
    const df y{lp[k].y, lp[k].ylo};
    const df x = df_mul(alpha, y);
    const df lx = df_log1p(x), ly = df_log1p(y);
    const df t = df_add(df_mul(df_add(df_make(1.0f), x), lx), df_neg(df_mul(x, df_add(df_make(1.0f), ly))));
    G = df_add(G, df_mul_f(t, lp[k].f));
    Gp = fmaf(lp[k].f * lp[k].y, lx.hi - ly.hi, Gp);
  }
}

// Forward pass of the 27-64-64-1 GELU network (weights in c_mlp).
__device__ __forceinline__ float fast_tanh(float u) {
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
  return t;
}
__device__ __forceinline__ float gelu_fast(float z) {
  return 0.5f * z * (1.0f + fast_tanh(0.7978845608028654f * fmaf(0.044715f * z * z, z, z)));
}
__device__ float mlp_forward(const float (&x)[Q]) {
  constexpr int NH = kMlpHidden, OB1 = Q * NH, OW2 = OB1 + NH, OB2 = OW2 + NH * NH, OW3 = OB2 + NH, OB3 = OW3 + NH;
  float h1[NH];
#pragma unroll
  for (int j = 0; j < NH; ++j) {
    float z = c_mlp[OB1 + j];
#pragma unroll
    for (int i = 0; i < Q; ++i) z = fmaf(x[i], c_mlp[i * NH + j], z);
    h1[j] = gelu_fast(z);
  }
  float out = c_mlp[OB3];
#pragma unroll 4
  for (int k = 0; k < NH; ++k) {
    float z = c_mlp[OB2 + k];
#pragma unroll
    for (int j = 0; j < NH; ++j) z = fmaf(h1[j], c_mlp[OW2 + j * NH + k], z);
    out = fmaf(gelu_fast(z), c_mlp[OW3 + k], out);
  }
  return out;
}

// g(2 + delta) and g'(2 + delta) of the truncated power series (see above).
template <int K>
__device__ __forceinline__ void series_g(const float (&S)[K + 1], float delta, float& g, float& gp) {
  // (P, alpha^(n-2)) and (g, g') advance as pairs on the paired FP32 pipe
  const float alpha = 2.0f + delta;
  const float2 aa = make_float2(alpha, alpha);
  float2 Pw = make_float2(0.f, 1.f);  // P_{n-2}, alpha^(n-2)
  float2 G = make_float2(0.f, 0.f);   // g, g'
  float two = 1.f;
#pragma unroll
  for (int n = 2; n <= K; ++n) {
    const float cgp = (float)(a_n(n) * (n - 1)) * Pw.y;
    Pw = __ffma2_rn(aa, Pw, make_float2(delta * two, 0.f));
    two *= 2.f;
    const float cg = fmaf((float)a_n(n), Pw.x, (float)c0_n(n));
    G = __ffma2_rn(make_float2(cg, cgp), make_float2(S[n], S[n]), G);
  }
  g = G.x;
  gp = G.y;
}

// Float-pair Newton over all 27 populations from alpha = 2: the fallback when
// the FP32 solve fails (rare; never in the hot loop).
__device__ __noinline__ bool df_newton_all(LargePop* lp, float amax, int max_it, float tol_dH, float& delta_hi,
                                           float& delta_lo, unsigned& iters) {
  df delta = df_make((2.0f < amax) ? 0.f : 0.5f * (amax - 3.0f));
  for (int it = 0; it < max_it; ++it) {
    df G;
    float Gp;
    df_terms(lp, Q, df_add(df_make(2.0f), delta), G, Gp);
    iters += 1;
    if (fabsf(G.hi) <= 0.25f * tol_dH) {
      delta_hi = delta.hi;
      delta_lo = delta.lo;
      return true;
    }
    if (!(Gp > 0.f)) {
      // left of the minimum of G (convex, G(0) = 0): towards the bracket's upper end, if it has one
      if (!(amax < INFINITY)) break;
      delta = df_make(0.5f * (delta.hi + amax - 2.0f));
      continue;
    }
    df next = df_add(delta, df_make(-G.hi / Gp));
    // a step that leaves the bracket (1, amax) is replaced by halving the way to its end (the
    // root can sit close to amax: a Newton step from the left overshoots it)
    if (!(2.0f + next.hi > 1.0f)) next = df_make(0.5f * (delta.hi - 1.0f));
    else if (!(2.0f + next.hi < amax)) next = df_make(0.5f * (delta.hi + amax - 2.0f));
    delta = next;
  }
  return false;
}

// The populations of one node as the alpha solve sees them: Delta (pairs),
// y = Delta / f (pairs), the deviations d = f - w.
struct NodePops {
  float2 D2[14], y2[14];
  float d[Q];
};

// Alpha solve of a node with strongly non-equilibrium populations
// (|y| > kYSmall; out of line, rare).  The other populations enter through
// their power sums; the strong ones add their truncated series for a first
// root, then Newton steps with their exact psi polish it (FP32), and a
// float-pair step follows where FP32 cannot resolve G to the tolerance.
template <int K>
__device__ __noinline__ AlphaOut alpha_solve_large(const NodePops& P, int max_it, float polish_thr, float tol_dH,
                                                   bool allow_df, float delta_start, int series_it) {
  const float2(&D2)[14] = P.D2;
  const float2(&y2)[14] = P.y2;
  const float(&d)[Q] = P.d;
  unsigned large = 0u;
  float ymin = 0.f;
#pragma unroll
  for (int q = 0; q < 14; ++q) {
    if (fabsf(y2[q].x) > kYSmall) large |= 1u << (2 * q);
    if (2 * q + 1 < Q && fabsf(y2[q].y) > kYSmall) large |= 1u << (2 * q + 1);
    ymin = fminf(ymin, fminf(y2[q].x, y2[q].y));
  }
  // positivity bracket: f + alpha Delta > 0 for all i  <=>  alpha < -1/min(y)
  const float amax = (ymin < 0.f) ? -1.0f / ymin : INFINITY;
  float2 S2[K + 1];
#pragma unroll
  for (int k = 0; k <= K; ++k) S2[k] = make_float2(0.f, 0.f);
#pragma unroll
  for (int q = 0; q < 14; ++q) {
    const bool sa = !(large & (1u << (2 * q))), sb = !(large & (1u << (2 * q + 1)));
    const float2 ym = make_float2(sa ? y2[q].x : 0.f, sb ? y2[q].y : 0.f);
    float2 p = __fmul2_rn(make_float2(sa ? D2[q].x : 0.f, sb ? D2[q].y : 0.f), ym);  // f y^2
    S2[2] = __fadd2_rn(S2[2], p);
#pragma unroll
    for (int k = 3; k <= K; ++k) {
      p = __fmul2_rn(p, ym);
      S2[k] = __fadd2_rn(S2[k], p);
    }
  }
  float S[K + 1];
#pragma unroll
  for (int k = 0; k <= K; ++k) S[k] = S2[k].x + S2[k].y;

  AlphaOut r{0.f, 0.f, 0u, large != 0u, false};
  LargePop lp[Q];
  int nl = 0;
  float SL[K + 1];
#pragma unroll
  for (int k = 0; k <= K; ++k) SL[k] = S[k];
  if (large) {
    // compact list (static indexing keeps the pair arrays in registers)
#pragma unroll
    for (int q = 0; q < 14; ++q) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int i = 2 * q + h;
        if (i < Q && (large & (1u << i))) {
          const float f = (float)w27(i) + d[i], D = h ? D2[q].y : D2[q].x, y = h ? y2[q].y : y2[q].x;
          lp[nl].f = f;
          lp[nl].y = y;
          lp[nl].ylo = __fdiv_rn(fmaf(-y, f, D), f);
          ++nl;
        }
      }
    }
    // their truncated series joins the first solve
    for (int k2 = 0; k2 < nl; ++k2) {
      const float y = lp[k2].y;
      float p = lp[k2].f * y * y;
      SL[2] += p;
#pragma unroll
      for (int k = 3; k <= K; ++k) {
        p *= y;
        SL[k] += p;
      }
    }
  }
  if (nl == 0 && !(S[2] > 1e-30f)) return r;  // at equilibrium: alpha = 2
  float delta = delta_start;
  bool ok = false;
  const int n_series = (series_it > 0) ? series_it : max_it;
  for (int it = 0; it < n_series; ++it) {
    float g, gp;
    series_g<K>(SL, delta, g, gp);
    r.iters = it + 1;
    if (!(gp > 0.f)) break;
    const float step = g / gp;
    const float next = delta - step;
    if (!(2.0f + next > 1.0f) || !(2.0f + next < amax)) break;
    delta = next;
    // Newton converges quadratically: the error left after this step is about
    // |g''/(2g')| step^2 <= (max|y|/3) step^2 <= 0.034 step^2 for the series
    // (g' ~ S_2/2, g'' ~ -S_3/3), below FP32 resolution once |step| <= 2e-4 |delta|
    if (fabsf(step) <= fmaxf(4e-8f, 2e-4f * fabsf(delta))) {
      ok = true;
      break;
    }
  }
  float gsmall = 0.f, gp_last = 0.f, GLabs = 0.f;
  if (ok && nl) {
    ok = false;
    for (int it = 0; it < 4; ++it) {
      const float alpha = 2.0f + delta;
      float g, gp, GL, GLp;
      series_g<K>(S, delta, g, gp);
      gsmall = g;
      large_terms(lp, nl, alpha, delta, GL, GLp, GLabs);
      const float ia = 1.0f / alpha;
      g = fmaf(GL, ia, g);
      gp += (GLp - GL * ia) * ia;
      gp_last = gp;
      r.iters += 1;
      if (!(gp > 0.f)) break;
      const float step = g / gp;
      const float next = delta - step;
      if (!(2.0f + next > 1.0f) || !(2.0f + next < amax)) break;
      delta = next;
      if (fabsf(step) <= fmaxf(4e-8f, 2e-7f * fabsf(delta))) {
        ok = true;
        break;
      }
    }
  }
  if (ok && nl && GLabs > polish_thr) {
    // FP32 cannot resolve G_L to the tolerance (its rounding error is ~1e-7 GLabs): Newton
    // steps with G_L in float pairs, the series part (accurate) in FP32, until |G| meets the
    // tolerance (at most three; otherwise the float-pair solve over all populations below)
    df dl = df_make(delta);
    ok = false;
    for (int pit = 0; pit < 3; ++pit) {
      float g, gp;
      series_g<K>(S, dl.hi, g, gp);
      const df alpha = df_add(df_make(2.0f), dl);
      df G;
      float Gp;
      df_terms(lp, nl, alpha, G, Gp);
      G = df_add(G, df_mul_f(alpha, g));  // G = alpha g_small + G_L
      r.iters += 1;
      if (fabsf(G.hi) <= 0.25f * tol_dH) {
        ok = true;
        break;
      }
      const float Gd = fmaf(alpha.hi, gp, g) + Gp;  // dG/dalpha = g_small + alpha g_small' + G_L'
      if (!(Gd > 0.f)) break;
      const df next = df_add(dl, df_make(-G.hi / Gd));
      if (!(2.0f + next.hi > 1.0f) || !(2.0f + next.hi < amax)) break;
      dl = next;
    }
    delta = dl.hi;
    r.delta_lo = ok ? dl.lo : 0.f;
    (void)gsmall;
    (void)gp_last;
  }
  if (!ok && allow_df) {
    // float-pair Newton over all populations; alpha = 2 (or inside the bracket) if that fails too
    nl = 0;
#pragma unroll
    for (int q = 0; q < 14; ++q) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int i = 2 * q + h;
        if (i < Q) {
          const float f = (float)w27(i) + d[i], D = h ? D2[q].y : D2[q].x, y = h ? y2[q].y : y2[q].x;
          lp[i].f = f;
          lp[i].y = y;
          lp[i].ylo = __fdiv_rn(fmaf(-y, f, D), f);
        }
      }
    }
    float hi = 0.f, lo = 0.f;
    if (df_newton_all(lp, amax, max_it, tol_dH, hi, lo, r.iters)) {
      delta = hi;
      r.delta_lo = lo;
    } else {
      r.fallback = true;
      delta = (2.0f < amax) ? 0.f : 0.5f * (amax - 3.0f);
    }
  } else if (!ok) {
    r.fallback = true;
    delta = (2.0f < amax) ? 0.f : 0.5f * (amax - 3.0f);
  }
  r.delta = delta;
  return r;
}

// Float-pair Newton over all populations for a node whose FP32 series solve
// failed (out of line, rare).
__device__ __noinline__ AlphaOut alpha_fallback(const NodePops& P, int max_it, float tol_dH, unsigned iters) {
  LargePop lp[Q];
  float ymin = 0.f;
#pragma unroll
  for (int q = 0; q < 14; ++q)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int i = 2 * q + h;
      if (i < Q) {
        const float f = (float)w27(i) + P.d[i], D = h ? P.D2[q].y : P.D2[q].x, y = h ? P.y2[q].y : P.y2[q].x;
        lp[i].f = f;
        lp[i].y = y;
        lp[i].ylo = __fdiv_rn(fmaf(-y, f, D), f);
        ymin = fminf(ymin, y);
      }
    }
  const float amax = (ymin < 0.f) ? -1.0f / ymin : INFINITY;
  AlphaOut r{0.f, 0.f, iters, false, false};
  float hi = 0.f, lo = 0.f;
  if (df_newton_all(lp, amax, max_it, tol_dH, hi, lo, r.iters)) {
    r.delta = hi;
    r.delta_lo = lo;
  } else {
    r.fallback = true;
    r.delta = (2.0f < amax) ? 0.f : 0.5f * (amax - 3.0f);
  }
  return r;
}

// Newton on the series g(2 + delta) from delta (at most n iterations) for a
// node whose populations all have |y| <= kYSmall.  Returns whether it converged.
template <int K>
__device__ __forceinline__ bool series_newton(const float (&S)[K + 1], int n, float& delta, unsigned& iters) {
  for (int it = 0; it < n; ++it) {
    float g, gp;
    series_g<K>(S, delta, g, gp);
    iters = it + 1;
    if (!(gp > 0.f)) return false;
    const float step = __fdividef(g, gp);
    const float next = delta - step;
    // every |y| <= 0.1 puts the positivity bracket at alpha >= 10
    if (!(next > -1.0f) || !(next < 8.0f)) return false;
    delta = next;
    // quadratic convergence: the error left is <= 0.034 step^2 (see alpha_solve_large)
    if (fabsf(step) <= fmaxf(4e-8f, 2e-4f * fabsf(delta))) return true;
  }
  return false;
}

// The alpha solve of one node.  Populations come in pairs (float2) so that the
// power sums run on the paired FP32 pipe.  ymax = max |y|.  Nodes with every
// |y| <= kYSmall (nearly all) take the inline series path below; the others
// the out-of-line solver above.
template <int K>
__device__ __forceinline__ AlphaOut alpha_solve32(const float2 (&D2)[14], const float2 (&y2)[14], const float (&d)[Q],
                                                  float ymax, int max_it, float polish_thr, float tol_dH,
                                                  bool allow_df = true, float delta_start = 0.f, int series_it = -1) {
  if (ymax > kYSmall) {
    NodePops P;
#pragma unroll
    for (int q = 0; q < 14; ++q) {
      P.D2[q] = D2[q];
      P.y2[q] = y2[q];
    }
#pragma unroll
    for (int i = 0; i < Q; ++i) P.d[i] = d[i];
    return alpha_solve_large<K>(P, max_it, polish_thr, tol_dH, allow_df, delta_start, series_it);
  }
  float2 S2[K + 1];
#pragma unroll
  for (int k = 0; k <= K; ++k) S2[k] = make_float2(0.f, 0.f);
#pragma unroll
  for (int q = 0; q < 14; ++q) {
    float2 p = __fmul2_rn(D2[q], y2[q]);  // f y^2  (the unused 28th lane holds 0)
    S2[2] = __fadd2_rn(S2[2], p);
#pragma unroll
    for (int k = 3; k <= K; ++k) {
      p = __fmul2_rn(p, y2[q]);
      S2[k] = __fadd2_rn(S2[k], p);
    }
  }
  float S[K + 1];
#pragma unroll
  for (int k = 0; k <= K; ++k) S[k] = S2[k].x + S2[k].y;
  AlphaOut r{0.f, 0.f, 0u, false, false};
  if (!(S[2] > 1e-30f)) return r;  // at equilibrium: alpha = 2
  float delta = delta_start;
  const bool ok = series_newton<K>(S, (series_it > 0) ? series_it : max_it, delta, r.iters);
  if (ok) {
    r.delta = delta;
    return r;
  }
  if (!allow_df) {
    r.fallback = true;
    return r;
  }
  NodePops P;
#pragma unroll
  for (int q = 0; q < 14; ++q) {
    P.D2[q] = D2[q];
    P.y2[q] = y2[q];
  }
#pragma unroll
  for (int i = 0; i < Q; ++i) P.d[i] = d[i];
  return alpha_fallback(P, max_it, tol_dH, r.iters);
}

// Moments and the factors of the entropic equilibrium of one node (from its
// deviations d): Delta_i follows from them with three operations.
struct NodeEq {
  float dr, rp1;     // rho - 1, rho
  float e0[3];       // per-axis factor minus one, x axis, c = -1, 0, +1
  float qyz[3][3];   // (y, z) part of prod(1 + e) - 1
  bool bad;          // rho or u not finite
};

__device__ __forceinline__ void node_eq(const float (&d)[Q], NodeEq& q) {
  // moments of the deviations: rho = 1 + sum d, j = sum c d (sum c w = 0), each as two
  // interleaved partial sums on the paired FP32 pipe (shorter dependency chains)
  float2 r2 = make_float2(0.f, 0.f), x2 = r2, y2 = r2, z2 = r2;
#pragma unroll
  for (int q2 = 0; q2 < 14; ++q2) {
    const int i0 = 2 * q2, i1 = 2 * q2 + 1;
    const float b = (i1 < Q) ? d[i1] : 0.f;
    const float2 v = make_float2(d[i0], b);
    r2 = __fadd2_rn(r2, v);
    if (cx27(i0) || (i1 < Q && cx27(i1)))
      x2 = __ffma2_rn(make_float2((float)cx27(i0), i1 < Q ? (float)cx27(i1) : 0.f), v, x2);
    if (cy27(i0) || (i1 < Q && cy27(i1)))
      y2 = __ffma2_rn(make_float2((float)cy27(i0), i1 < Q ? (float)cy27(i1) : 0.f), v, y2);
    if (cz27(i0) || (i1 < Q && cz27(i1)))
      z2 = __ffma2_rn(make_float2((float)cz27(i0), i1 < Q ? (float)cz27(i1) : 0.f), v, z2);
  }
  const float dr = r2.x + r2.y, jx = x2.x + x2.y, jy = y2.x + y2.y, jz = z2.x + z2.y;
  const float rho = 1.0f + dr;
  const float inv_rho = __fdividef(1.0f, rho);
  const float u[3] = {jx * inv_rho, jy * inv_rho, jz * inv_rho};
  // per-axis factor of the entropic equilibrium relative to its weight, minus one:
  // e_0 = psi - 1, e_+ = psi*zeta - 1, e_- = psi/zeta - 1, from small quantities only
  // (quotients of well-scaled operands near 1: the fast reciprocal-based division)
  float e[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float uu = u[k] * u[k];
    const float sm1 = __fdividef(3.0f * uu, 1.0f + sqrtf(fmaf(3.0f, uu, 1.0f)));  // sqrt(1+3u^2) - 1
    const float zm1 = __fdividef(3.0f * u[k] + sm1, 1.0f - u[k]);                 // zeta - 1
    e[k][1] = -sm1;
    e[k][2] = fmaf(1.0f - sm1, zm1, -sm1);
    e[k][0] = __fdividef(-sm1 - zm1, 1.0f + zm1);
  }
  // P_i = prod(1 + e) - 1 = A + (1 + A)(B + (1 + B) C), with the (y, z) part shared
#pragma unroll
  for (int b = 0; b < 3; ++b)
#pragma unroll
    for (int c = 0; c < 3; ++c) q.qyz[b][c] = fmaf(1.0f + e[1][b], e[2][c], e[1][b]);
#pragma unroll
  for (int c = 0; c < 3; ++c) q.e0[c] = e[0][c];
  q.dr = dr;
  q.rp1 = 1.0f + dr;
  q.bad = !isfinite(rho) || !isfinite(u[0]) || !isfinite(u[1]) || !isfinite(u[2]);
}

// Delta_i = f^eq_i - f_i in deviation form, w_i [P (1 + dr) + dr] - d_i, for the
// pair (2q, 2q + 1) (the 28th lane is 0).
__device__ __forceinline__ float2 delta_pair(const NodeEq& e, const float (&d)[Q], int q) {
  float v[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int i = 2 * q + h;
    if (i < Q) {
      const float A = e.e0[cx27(i) + 1];
      const float P = fmaf(1.0f + A, e.qyz[cy27(i) + 1][cz27(i) + 1], A);
      v[h] = fmaf((float)w27(i), fmaf(P, e.rp1, e.dr), -d[i]);
    } else {
      v[h] = 0.f;
    }
  }
  return make_float2(v[0], v[1]);
}

// f = w + d for the pair (2q, 2q + 1) (the 28th lane is 1).
__device__ __forceinline__ float2 f_pair(const float (&d)[Q], int q) {
  return make_float2((float)w27(2 * q) + d[2 * q], (2 * q + 1 < Q) ? (float)w27(2 * q + 1) + d[2 * q + 1] : 1.0f);
}

// Moments, entropic equilibrium and Delta = f^eq - f of one node from its
// deviations d (pairs D2); with want_y, also y = Delta / f (pairs y2) and
// ymax = max |y|.  bad: rho or u not finite.
__device__ __forceinline__ void node_prepare(const float (&d)[Q], bool want_y, float2 (&D2)[14], float2 (&y2)[14],
                                             float& ymax, bool& bad) {
  NodeEq e;
  node_eq(d, e);
#pragma unroll
  for (int q = 0; q < 14; ++q) D2[q] = delta_pair(e, d, q);
  bad = e.bad;
  ymax = 0.f;
  if (want_y) {
#pragma unroll
    for (int q = 0; q < 14; ++q) {
      const float2 f2 = f_pair(d, q);
      y2[q] = make_float2(__fdividef(D2[q].x, f2.x), __fdividef(D2[q].y, f2.y));
      ymax = fmaxf(ymax, fmaxf(fabsf(y2[q].x), fabsf(y2[q].y)));
    }
  }
}

// Alpha solve (from delta0 with at most series_it series steps when
// series_it > 0, the learned guess), relaxation, store and statistics.
template <bool CHECK, int MODE, bool ACC = false>
__device__ __forceinline__ void node_finish(const Step27Args& a, int64_t n, float (&d)[Q], const float2 (&D2)[14],
                                            const float2 (&y2)[14], float ymax, bool bad, float delta0,
                                            int series_it, StatAcc* acc = nullptr) {
  float* __restrict__ dst = static_cast<float*>(a.dst);
  AlphaOut al{0.f, 0.f, 0u, false, false};
  double dH = 0.0;
  bool guess_miss = false;
  if (a.alpha_mode != 0) {
    const float lam = ymax;
    // float-pair polish above this error scale (the FP32 rounding of G_L stays below ~5e-7 GLabs)
    const float pthr = (float)(a.tol_dH * 1e6), tdh = (float)a.tol_dH;
    al = alpha_solve32<kSeriesK>(D2, y2, d, ymax, a.max_newton, pthr, tdh, MODE != 1, delta0, series_it);
    if (MODE == 1 && al.fallback) {
      // the guess did not converge in two steps: plain Newton from alpha = 2
      guess_miss = true;
      const unsigned it0 = al.iters;
      al = alpha_solve32<kSeriesK>(D2, y2, d, ymax, a.max_newton, pthr, tdh);
      al.iters += it0;
    }
    if (MODE == 2 && !al.fallback && lam > 0.f && (n % a.harvest_stride) == 0) {
      const unsigned long long slot = atomicAdd(a.harvest_count, 1ull);
      if ((long long)slot < a.harvest_cap) {
        float* r = a.harvest + slot * kMlpRecord;
        const float il = 1.0f / lam;
#pragma unroll
        for (int i = 0; i < Q; ++i) r[i] = ((i & 1) ? y2[i >> 1].y : y2[i >> 1].x) * il;
        r[Q] = lam;
        r[Q + 1] = al.delta * il;
      }
    }
    if (CHECK) {
      // |H(f + alpha Delta) - H(f)| in FP64 (conservation-consistent form) from the FP32 populations
      const double al64 = 2.0 + (double)al.delta + (double)al.delta_lo;
      double g = 0.0;
#pragma unroll
      for (int i = 0; i < Q; ++i) {
        const double f64 = (double)((float)w27(i) + d[i]);
        const double y64 = (double)((i & 1) ? D2[i >> 1].y : D2[i >> 1].x) / f64;
        g += f64 * (phi64(al64 * y64) - al64 * y64 * log1p(y64));
      }
      dH = fabs(g);
    }
  }
  unsigned flags = 0;
  if (bad) flags |= 0x1u;
  if (al.fallback) flags |= 0x2u;
  if (CHECK && dH > a.tol_dH) flags |= 0x8u;
  const float ab = (2.0f + al.delta) * (float)a.beta;
  bool neg = false;
  const float2 ab2 = make_float2(ab, ab);
#pragma unroll
  for (int q = 0; q < 13; ++q) {
    const float2 r = __ffma2_rn(ab2, D2[q], make_float2(d[2 * q], d[2 * q + 1]));
    d[2 * q] = r.x;
    d[2 * q + 1] = r.y;
  }
  d[26] = fmaf(ab, D2[13].x, d[26]);
  // f = w + d < 0, compared without forming the sum (same outcome without flush-to-zero)
#pragma unroll
  for (int i = 0; i < Q; ++i) neg |= d[i] < -(float)w27(i);
  if (neg) flags |= 0x4u;
  if (neg && a.neg_list) {
#pragma unroll
    for (int i = 0; i < Q; ++i)
      if (d[i] < -(float)w27(i)) {
        const unsigned long long slot = atomicAdd(a.neg_count, 1ull);
        if ((long long)slot < a.neg_cap) a.neg_list[slot] = (unsigned long long)n * Q + i;
      }
  }
  store_dst(dst, a.plane, n, d);
  if (a.alpha_out) a.alpha_out[n] = 2.0f + al.delta;
  if constexpr (ACC) {
    acc->nodes_exact += 1u + (al.large ? 0x10000u : 0u);
    acc->fb_over += (al.fallback ? 1u : 0u) + ((flags & 0x8u) ? 0x10000u : 0u);
    acc->iters += al.iters;
    acc->flags |= flags;
    if (CHECK) acc->dH = fmax(acc->dH, dH);
  } else {
    warp_stats(a.stats, true, al.iters, al.large, al.fallback, flags, dH);
  }
  if (MODE == 1) {
    const unsigned mk = __activemask();
    const unsigned nm = __popc(__ballot_sync(mk, guess_miss));
    if (nm && (int)(threadIdx.x & 31) == __ffs(mk) - 1) atomicAdd(&a.stats->guess_misses, (unsigned long long)nm);
  }
}

// Everything after the gather: moments, equilibrium, alpha, relaxation, store.
// The out-of-line solvers on a node given by its deviations alone (Delta and
// y formed again, exactly as node_prepare forms them).
__device__ __noinline__ AlphaOut alpha_solve_from_d(NodePops& P, int max_it, float polish_thr, float tol_dH,
                                                    bool series_failed, unsigned iters) {
  float ymax;
  bool bad;
  node_prepare(P.d, true, P.D2, P.y2, ymax, bad);
  if (series_failed) return alpha_fallback(P, max_it, tol_dH, iters);
  return alpha_solve_large<kSeriesK>(P, max_it, polish_thr, tol_dH, true, 0.f, -1);
}

// The Newton-alpha update of one node with little live state: the
// equilibrium factors (NodeEq) stay, while each pair of Delta and y is formed,
// added into the power sums and dropped; the relaxation forms Delta again
// (the same operations, so the same values).  Nodes with some |y| > kYSmall go
// to the out-of-line solver, or, with a deferred-node list, to the second
// kernel.
template <bool CHECK, bool ACC>
__device__ __forceinline__ void node_update_newton(const Step27Args& a, int64_t n, float (&d)[Q], StatAcc* acc) {
  constexpr int K = kSeriesK;
  NodeEq e;
  node_eq(d, e);
  AlphaOut al{0.f, 0.f, 0u, false, false};
  if (a.alpha_mode != 0) {
    float ymax = 0.f;
    float2 S2[K + 1];
#pragma unroll
    for (int k = 0; k <= K; ++k) S2[k] = make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 14; ++q) {
      const float2 D = delta_pair(e, d, q), f2 = f_pair(d, q);
      const float2 y = make_float2(__fdividef(D.x, f2.x), __fdividef(D.y, f2.y));
      ymax = fmaxf(ymax, fmaxf(fabsf(y.x), fabsf(y.y)));
      float2 p = __fmul2_rn(D, y);  // f y^2
      S2[2] = __fadd2_rn(S2[2], p);
#pragma unroll
      for (int k = 3; k <= K; ++k) {
        p = __fmul2_rn(p, y);
        S2[k] = __fadd2_rn(S2[k], p);
      }
    }
    if (a.defer_on) {
      // a node whose populations leave the series range takes the out-of-line solver, which would
      // hold its whole warp: list it for the second kernel instead (warp-aggregated slots)
      const bool defer = ymax > kYSmall;
      const unsigned mk = __activemask();
      const unsigned dm = __ballot_sync(mk, defer);
      if (dm) {
        const int lane = (int)(threadIdx.x & 31), leader = __ffs(dm) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(a.defer_count, (unsigned long long)__popc(dm));
        base = __shfl_sync(mk, base, leader);
        if (defer) {
          const unsigned long long slot = base + __popc(dm & ((1u << lane) - 1u));
          if ((long long)slot < a.defer_cap) {
            a.defer_list[slot] = (uint32_t)n;
            return;
          }
        }
      }
    }
    const float pthr = (float)(a.tol_dH * 1e6), tdh = (float)a.tol_dH;
    bool need_pops = ymax > kYSmall, series_failed = false;
    if (!need_pops) {
      float S[K + 1];
#pragma unroll
      for (int k = 0; k <= K; ++k) S[k] = S2[k].x + S2[k].y;
      if (S[2] > 1e-30f) {  // else at equilibrium: alpha = 2
        float delta = 0.f;
        if (series_newton<K>(S, a.max_newton, delta, al.iters)) al.delta = delta;
        else need_pops = series_failed = true;
      }
    }
    if (need_pops) {
      NodePops P;
#pragma unroll
      for (int i = 0; i < Q; ++i) P.d[i] = d[i];
      al = alpha_solve_from_d(P, a.max_newton, pthr, tdh, series_failed, al.iters);
    }
  }
  double dH = 0.0;
  if (CHECK && a.alpha_mode != 0) {
    // |H(f + alpha Delta) - H(f)| in FP64 (conservation-consistent form) from the FP32 populations
    const double al64 = 2.0 + (double)al.delta + (double)al.delta_lo;
    double g = 0.0;
#pragma unroll
    for (int q = 0; q < 14; ++q) {
      const float2 D = delta_pair(e, d, q), f2 = f_pair(d, q);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (2 * q + h < Q) {
          const double f64 = (double)(h ? f2.y : f2.x);
          const double y64 = (double)(h ? D.y : D.x) / f64;
          g += f64 * (phi64(al64 * y64) - al64 * y64 * log1p(y64));
        }
      }
    }
    dH = fabs(g);
  }
  unsigned flags = 0;
  if (e.bad) flags |= 0x1u;
  if (al.fallback) flags |= 0x2u;
  if (CHECK && dH > a.tol_dH) flags |= 0x8u;
  const float ab = (2.0f + al.delta) * (float)a.beta;
  const float2 ab2 = make_float2(ab, ab);
  // d += alpha beta Delta (Delta formed again)
#pragma unroll
  for (int q = 0; q < 14; ++q) {
    const float2 D = delta_pair(e, d, q);
    if (2 * q + 1 < Q) {
      const float2 r = __ffma2_rn(ab2, D, make_float2(d[2 * q], d[2 * q + 1]));
      d[2 * q] = r.x;
      d[2 * q + 1] = r.y;
    } else {
      d[2 * q] = fmaf(ab, D.x, d[2 * q]);
    }
  }
  // f = w + d < 0, compared without forming the sum (same outcome without flush-to-zero)
  bool neg = false;
#pragma unroll
  for (int i = 0; i < Q; ++i) neg |= d[i] < -(float)w27(i);
  if (neg) flags |= 0x4u;
  if (neg && a.neg_list) {
#pragma unroll
    for (int i = 0; i < Q; ++i)
      if (d[i] < -(float)w27(i)) {
        const unsigned long long slot = atomicAdd(a.neg_count, 1ull);
        if ((long long)slot < a.neg_cap) a.neg_list[slot] = (unsigned long long)n * Q + i;
      }
  }
  store_dst(static_cast<float*>(a.dst), a.plane, n, d);
  if (a.alpha_out) a.alpha_out[n] = 2.0f + al.delta;
  if constexpr (ACC) {
    acc->nodes_exact += 1u + (al.large ? 0x10000u : 0u);
    acc->fb_over += (al.fallback ? 1u : 0u) + ((flags & 0x8u) ? 0x10000u : 0u);
    acc->iters += al.iters;
    acc->flags |= flags;
    if (CHECK) acc->dH = fmax(acc->dH, dH);
  } else {
    warp_stats(a.stats, true, al.iters, al.large, al.fallback, flags, dH);
  }
}

template <bool CHECK, int MODE, bool ACC = false>
__device__ __forceinline__ void node_update(const Step27Args& a, int64_t n, float (&d)[Q], StatAcc* acc = nullptr) {
  if constexpr (MODE == 0) {
    node_update_newton<CHECK, ACC>(a, n, d, acc);
    return;
  }
  float2 D2[14], y2[14];
  float ymax;
  bool bad;
  node_prepare(d, a.alpha_mode != 0, D2, y2, ymax, bad);
  if (MODE != 1 && a.defer_on && a.alpha_mode != 0) {
    // a node whose populations leave the series range takes the out-of-line solver, which would
    // hold its whole warp: list it for the second kernel instead (warp-aggregated slots)
    const bool defer = ymax > kYSmall;
    const unsigned mk = __activemask();
    const unsigned dm = __ballot_sync(mk, defer);
    if (dm) {
      const int lane = (int)(threadIdx.x & 31), leader = __ffs(dm) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(a.defer_count, (unsigned long long)__popc(dm));
      base = __shfl_sync(mk, base, leader);
      if (defer) {
        const unsigned long long slot = base + __popc(dm & ((1u << lane) - 1u));
        if ((long long)slot < a.defer_cap) {
          a.defer_list[slot] = (uint32_t)n;
          return;
        }
      }
    }
  }
  float delta0 = 0.f;
  int series_it = -1;
  if (MODE == 1 && a.alpha_mode != 0 && ymax > 0.f) {
    // learned guess: alpha = 2 + lambda * net(y / lambda), then at most two Newton steps
    float x[Q];
    const float il = 1.0f / ymax;
#pragma unroll
    for (int i = 0; i < Q; ++i) x[i] = ((i & 1) ? y2[i >> 1].y : y2[i >> 1].x) * il;
    delta0 = ymax * mlp_forward(x);
    series_it = 2;
  }
  node_finish<CHECK, MODE, ACC>(a, n, d, D2, y2, ymax, bad, delta0, series_it, acc);
}

// MINB: minimum resident blocks per SM requested from the register allocator
// (0: none).  Both variants are built; the level's autotuner picks one.
// MODE 0: Newton from alpha = 2; 1: learned guess + at most two Newton steps,
// Newton from 2 as the fallback; 2: Newton and harvesting of training records.
// Direct variant: one thread per node, the 27 pulls are plain global loads.
template <bool CHECK, int MINB, int MODE = 0, bool OFF = false>
__global__ void __launch_bounds__(128, MINB) d3q27_fp32_kernel(const Step27Args a) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.N) return;
  // bulk nodes only: the boundary nodes are the boundary kernel's
  if (__ldg(a.ntype + n) != NT_BULK) return;
  float d[Q];
  if constexpr (OFF) gather_bulk_off(a, static_cast<const float*>(a.src), n, d);
  else gather_bulk(a, static_cast<const float*>(a.src), n, d);
  node_update<CHECK, MODE>(a, n, d);
}

// The listed nodes of a step (strongly non-equilibrium ones), one thread each:
// the same gather and update as in the step kernel, so that a node's result
// does not depend on where it is finished.  A fixed grid strides over the list.
template <bool CHECK, int MODE>
__global__ void __launch_bounds__(128) d3q27_fp32_deferred_kernel(const Step27Args a) {
  const unsigned long long cnt = *a.defer_count;
  const long long m = (long long)cnt < a.defer_cap ? (long long)cnt : a.defer_cap;
  Step27Args b = a;
  b.defer_on = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x) {
    const int64_t n = a.defer_list[i];
    const uint8_t t = __ldg(a.ntype + n);
    float d[Q];
    gather(b, static_cast<const float*>(b.src), n, t, d);
    node_update<CHECK, MODE>(b, n, d);
  }
}

// The boundary nodes of a step (the records' nodes), one thread each: their
// pulls follow the link words; the update is the bulk nodes' (nodes far from
// equilibrium are solved in place).
template <bool CHECK, int MODE>
__global__ void __launch_bounds__(128) d3q27_fp32_boundary_kernel(const Step27Args a) {
  Step27Args b = a;
  b.defer_on = 0;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < a.nbnd;
       r += (long long)gridDim.x * blockDim.x) {
    const int64_t n = __ldg(a.bnode + r);
    float d[Q];
    if (a.rsrc) gather_resolved(b, static_cast<const float*>(b.src), n, (int32_t)r, d);
    else gather(b, static_cast<const float*>(b.src), n, (uint8_t)NT_BOUNDARY, d, (int32_t)r);
    node_update<CHECK, MODE>(b, n, d);
  }
}

// Persistent variant: a fixed grid (every SM full) whose warps take chunks of
// 32 consecutive nodes from a global counter, in order, so that no block waits
// for its slowest warp before the SM can start new work and the chunks in
// flight stay close together in memory.
template <bool CHECK, int MINB, int MODE = 0>
__global__ void __launch_bounds__(128, MINB) d3q27_fp32_persistent_kernel(const Step27Args a) {
  const int64_t nchunks = (a.N + 31) / 32;
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long c = 0;
    if (lane == 0) c = atomicAdd(a.work_counter, 1ull);
    c = __shfl_sync(0xffffffffu, c, 0);
    if ((int64_t)c >= nchunks) break;
    const int64_t n = (int64_t)c * 32 + lane;
    if (n >= a.N) continue;
    if (__ldg(a.ntype + n) != NT_BULK) continue;  // the boundary kernel updates the others
    float d[Q];
    gather_bulk(a, static_cast<const float*>(a.src), n, d);
    node_update<CHECK, MODE>(a, n, d);
  }
}

// ---------------------------------------------------------------------------
// Staged variant: a persistent CTA walks tiles of kTileX nodes along x.  For
// a tile in an interior row, one thread issues 27 bulk copies (one per
// population: the row segment the pull reads, x0-4 .. x0+kTileX+4) into a
// shared-memory stage tracked by an mbarrier; kStages tiles are in flight
// while the CTA computes, so the HBM traffic no longer waits on the
// per-thread register budget.  Bulk nodes read their pulls from shared
// memory; boundary nodes use the link-word gather from global memory.
// ---------------------------------------------------------------------------
constexpr int kTileX = 128, kHalo = 4, kSegLen = kTileX + 2 * kHalo, kStages = 2;
constexpr int kStageFloats = Q * kSegLen;
constexpr unsigned kStageBytes = kStageFloats * 4;
// Bounded mbarrier waits: each poll may suspend the thread for a short,
// hardware-chosen time, and a wait gives up after 2^20 polls or 2 s of the
// global timer, whichever first.
constexpr int kSpinLimit = 1 << 20;
constexpr unsigned long long kWaitLimitNs = 2000000000ull;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const unsigned long long t0 = global_ns();
  for (int i = 0; i < kSpinLimit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if ((i & 255) == 255 && global_ns() - t0 > kWaitLimitNs) return false;
  }
  return false;
}

// Issue the copies of one tile into one stage (one thread).  Returns false for
// tiles whose row touches the box faces: all their nodes are boundary nodes.
__device__ __forceinline__ void issue_tile(const Step27Args& a, const float* src, int64_t tile, int tiles_x,
                                           float* stage, uint32_t bar) {
  const int tx = (int)(tile % tiles_x);
  const int64_t row = tile / tiles_x;
  const int y = (int)(row % a.ny), z = (int)(row / a.ny);
  const bool interior = y >= 1 && y <= a.ny - 2 && z >= 1 && z <= a.nz - 2;
  const unsigned tx_bytes = interior ? kStageBytes : 0u;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(tx_bytes) : "memory");
  if (!interior) return;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  const int64_t x0 = (int64_t)tx * kTileX;
#pragma unroll 1
  for (int j = 0; j < Q; ++j) {
    const float* g = src + (int64_t)j * a.plane + ((int64_t)(z - cz27(j)) * a.ny + (y - cy27(j))) * a.nx + x0 - kHalo;
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(stage + j * kSegLen)),
        "l"(g), "r"((unsigned)(kSegLen * 4)), "r"(bar)
        : "memory");
  }
}

template <bool CHECK, int MODE = 0>
__global__ void __launch_bounds__(128, 3) d3q27_fp32_staged_kernel(const Step27Args a) {
  extern __shared__ __align__(128) float sm[];
  __shared__ __align__(8) unsigned long long bars[kStages];
  const float* __restrict__ src = static_cast<const float*>(a.src);
  const int tiles_x = (a.nx + kTileX - 1) / kTileX;
  const int64_t ntiles = (int64_t)tiles_x * a.ny * a.nz;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[s])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int s = 0; s < kStages; ++s) {
      const int64_t tile = blockIdx.x + (int64_t)s * gridDim.x;
      if (tile < ntiles) issue_tile(a, src, tile, tiles_x, sm + s * kStageFloats, smem_addr(&bars[s]));
    }
  }
  __syncthreads();
  int64_t it = 0;
  bool failed = false;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int s = (int)(it % kStages);
    const bool ok = mbar_wait(smem_addr(&bars[s]), (uint32_t)((it / kStages) & 1));
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    const int tx = (int)(tile % tiles_x);
    const int64_t row = tile / tiles_x;
    const int x = tx * kTileX + (int)threadIdx.x;
    const int64_t n = row * a.nx + x;
    const uint8_t t = x < a.nx ? __ldg(a.ntype + n) : (uint8_t)NT_SKIP;
    float d[Q];
    if (t == NT_BULK) {
      const float* stg = sm + s * kStageFloats + kHalo + threadIdx.x;
#pragma unroll
      for (int j = 0; j < Q; ++j) d[j] = stg[j * kSegLen - cx27(j)];
    }
    __syncthreads();  // every read of stage s is done: refill it
    if (threadIdx.x == 0) {
      const int64_t next = tile + (int64_t)kStages * gridDim.x;
      if (next < ntiles) issue_tile(a, src, next, tiles_x, sm + s * kStageFloats, smem_addr(&bars[s]));
    }
    if (t == NT_BULK) node_update<CHECK, MODE>(a, n, d);  // the boundary kernel updates the others
  }
  if (failed && threadIdx.x == 0) {
    // report, then wait (bounded) for this block's copies still in flight before the
    // shared memory they target is released
    atomicOr(&a.stats->status, (unsigned)ELBM_ST_COPY_TIMEOUT);
    for (int64_t k = it; k < it + kStages; ++k)
      if (blockIdx.x + k * gridDim.x < ntiles) mbar_wait(smem_addr(&bars[k % kStages]), (uint32_t)((k / kStages) & 1));
  }
}

// ---------------------------------------------------------------------------
// Tensor-copy variant.  A persistent CTA of eight warps walks 256-node tiles
// (TX x TY nodes of one z plane, TX in {32, 64, 128} by box width), one node
// per thread.  Per tile, one 4-D tensor copy (cp.async.bulk.tensor) per
// population j brings the box (x0 - 4 .. x0 + TX + 4, y0 - cy_j .. y0 - cy_j
// + TY, z - cz_j, j) of the source buffer into a stage of a kWsStages-deep
// shared-memory ring, completing on the stage's `full` mbarrier.  The x start
// is rounded to a 16-byte boundary (x0 - 4) and the x shift -cx_j is taken in
// shared memory; y and z shifts are tensor coordinates, so halo rows outside
// the box come as zero fill (only boundary nodes would pull from there, and
// they use their link words).  Each thread reads its 27 pulls from the stage
// at compile-time offsets and its warp releases the stage (one arrive on
// `empty`); one thread then refills the stage with the tile kWsStages ahead
// once all eight warps have released it, so copies of the next tiles are in
// flight while the current one computes.  The issuing thread is one of the
// consumers (no producer warp): eight warps per CTA and two CTAs per SM leave
// 128 registers per thread.  Every mbarrier wait is bounded: a wait that gives
// up sets ELBM_ST_COPY_TIMEOUT, and the issuing thread waits (bounded) for its
// copies still in flight before the CTA exits.
// ---------------------------------------------------------------------------
constexpr int kWsWarps = kWsTileNodes / 32;
constexpr int kWsThreads = 32 * kWsWarps;
constexpr int kWsStages = 3;
// floats per population in a stage: the largest TY (TX + 8) over the tile shapes
// (TX = 32: 8 x 40 = 320); 1,280 bytes keeps every copy's destination 128-byte aligned
constexpr int kWsPopStride = 320;
constexpr int kWsStageFloats = Q * kWsPopStride;

// Levels of up to kWsSmemBoxes boxes keep their tilings in shared memory.
constexpr int kWsSmemBoxes = 64;

struct WsSmem {
  float stage[kWsStages][kWsStageFloats];
  unsigned long long full[kWsStages];
  unsigned long long empty[kWsStages];
  WsBox boxes[kWsSmemBoxes];
};

// Box of a tile: the last box whose first tile is <= tile (binary search; one box: none).
__device__ __forceinline__ int ws_find_box(const WsBox* boxes, int nbox, int64_t tile) {
  int lo = 0, hi = nbox - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (boxes[mid].tile0 <= tile) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

struct WsTile {
  int box, tx_log2, x0, y0, z;
  int nx, ny;
  int64_t base;
};

// Tile coordinates (32-bit arithmetic: a level holds fewer than 2^31 nodes, so
// fewer tiles); `boxes` is the level's table (shared memory or global).
__device__ __forceinline__ WsTile ws_tile(const Step27Args& a, const WsBox* boxes, int tile) {
  WsTile t;
  t.box = (a.nbox > 1) ? ws_find_box(boxes, a.nbox, tile) : 0;
  const WsBox& b = boxes[t.box];
  const unsigned lt = (unsigned)(tile - (int)b.tile0);
  const unsigned tiles_x = (unsigned)b.tiles_x, tiles_y = (unsigned)b.tiles_y;
  t.tx_log2 = b.tx_log2;
  const unsigned row = lt / tiles_x;
  const unsigned zz = row / tiles_y;
  t.x0 = (int)(lt - row * tiles_x) << t.tx_log2;
  t.y0 = (int)(row - zz * tiles_y) * (kWsTileNodes >> t.tx_log2);
  t.z = (int)zz;
  t.nx = b.nx;
  t.ny = b.ny;
  t.base = b.base;
  return t;
}

// The node a consumer thread (ct = 0 .. 255) owns in a tile, and its type byte.
__device__ __forceinline__ uint8_t ws_node(const Step27Args& a, const WsTile& t, int ct, int& r, int& xl,
                                           int64_t& n) {
  const int TX = 1 << t.tx_log2;
  r = ct >> t.tx_log2;
  xl = ct & (TX - 1);
  const int x = t.x0 + xl, y = t.y0 + r;
  n = t.base + ((int64_t)t.z * t.ny + y) * t.nx + x;
  return (x < t.nx && y < t.ny) ? __ldg(a.ntype + n) : (uint8_t)NT_SKIP;
}

__device__ __forceinline__ void ws_tma_load(uint32_t dst, const void* map, int x, int y, int z, int j, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(j), "r"(bar)
      : "memory");
}

// The issuing thread's copies of one tile into stage s.
__device__ __forceinline__ void ws_issue(const Step27Args& a, WsSmem& S, const WsBox* boxes, int tile, int s) {
  const WsTile t = ws_tile(a, boxes, tile);
  const int TX = 1 << t.tx_log2, TY = kWsTileNodes >> t.tx_log2;
  const unsigned bytes = (unsigned)(Q * TY * (TX + 8) * 4);
  const uint32_t bar = smem_addr(&S.full[s]);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
  const void* map = static_cast<const unsigned char*>(a.ws_maps) + (size_t)t.box * 128;
  const uint32_t dst = smem_addr(&S.stage[s][0]);
#pragma unroll
  for (int j = 0; j < Q; ++j)
    ws_tma_load(dst + (uint32_t)(j * kWsPopStride * 4), map, t.x0 - 4, t.y0 - cy27(j), t.z - cz27(j), j, bar);
}

template <bool CHECK>
__global__ void __launch_bounds__(kWsThreads, 2) d3q27_fp32_ws_kernel(const Step27Args a) {
  extern __shared__ __align__(1024) unsigned char ws_raw[];
  WsSmem& S = *reinterpret_cast<WsSmem*>(ws_raw);
  const int lane = (int)(threadIdx.x & 31);
  const bool issuer = threadIdx.x == 0;
  const int ntiles = (int)a.ws_ntiles;
  // this CTA's tiles: blockIdx.x + k gridDim.x, k = 0 .. mine - 1
  const int mine = ((int)blockIdx.x < ntiles) ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  const bool smem_boxes = a.nbox <= kWsSmemBoxes;
  if (smem_boxes)
    for (int k = (int)threadIdx.x; k < a.nbox; k += (int)blockDim.x) S.boxes[k] = a.ws_boxes[k];
  const WsBox* boxes = smem_boxes ? S.boxes : a.ws_boxes;
  __syncthreads();
  if (issuer) {
    for (int s = 0; s < kWsStages; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&S.full[s])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&S.empty[s])), "r"(kWsWarps)
                   : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int k = 0; k < kWsStages && k < mine; ++k)
      ws_issue(a, S, boxes, (int)blockIdx.x + k * (int)gridDim.x, k);
  }
  __syncthreads();

  const int ct = (int)threadIdx.x;  // 0 .. 255: the node of the tile
  StatAcc acc;
  int issued = (mine < kWsStages) ? mine : kWsStages;
  bool failed = false;
  int tile = blockIdx.x;
  int r, xl;
  int64_t n;
  // the type byte of this thread's node in the next tile is loaded while the current one computes
  uint8_t nt_next = ws_node(a, ws_tile(a, boxes, tile), ct, r, xl, n);
  for (int it = 0; it < mine; ++it, tile += gridDim.x) {
    const int s = it % kWsStages;
    const uint32_t ph = (uint32_t)((it / kWsStages) & 1);
    const WsTile t = ws_tile(a, boxes, tile);
    const int TX = 1 << t.tx_log2;
    r = ct >> t.tx_log2;
    xl = ct & (TX - 1);
    n = t.base + ((int64_t)t.z * t.ny + t.y0 + r) * t.nx + t.x0 + xl;
    const uint8_t nt = nt_next;
    if (!__all_sync(0xffffffffu, mbar_wait(smem_addr(&S.full[s]), ph))) {
      failed = true;
      break;
    }
    float d[Q];
    if (nt == NT_BULK) {
      const float* p = &S.stage[s][r * (TX + 8) + xl + 4];
#pragma unroll
      for (int j = 0; j < Q; ++j) d[j] = p[j * kWsPopStride - cx27(j)];
    }
    __syncwarp();
    if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&S.empty[s])) : "memory");
    if (issuer && it + kWsStages < mine) {
      // every warp has read this tile's stage: refill it with the tile kWsStages ahead
      if (mbar_wait(smem_addr(&S.empty[s]), ph)) {
        ws_issue(a, S, boxes, (int)blockIdx.x + (it + kWsStages) * (int)gridDim.x, s);
        ++issued;
      } else {
        failed = true;
      }
    }
    if (__any_sync(0xffffffffu, failed)) {
      failed = true;
      break;
    }
    if (it + 1 < mine) {
      int r2, xl2;
      int64_t n2;
      nt_next = ws_node(a, ws_tile(a, boxes, tile + (int)gridDim.x), ct, r2, xl2, n2);
    }
    if (nt == NT_BULK) node_update<CHECK, 0, true>(a, n, d, &acc);  // the boundary kernel updates the others
  }
  __syncwarp();
  flush_stats(a.stats, acc);
  if (failed && lane == 0) atomicOr(&a.stats->status, (unsigned)ELBM_ST_COPY_TIMEOUT);
  if (issuer) {
    // the copies of the last issued tiles must land before the CTA's shared memory is released
    for (int k = (issued > kWsStages ? issued - kWsStages : 0); k < issued; ++k)
      mbar_wait(smem_addr(&S.full[k % kWsStages]), (uint32_t)((k / kWsStages) & 1));
  }
}

}  // namespace

void launch_d3q27_fp64(const Step27Args& a, cudaStream_t s) {
  const int threads = 128;
  const int64_t blocks = (a.N + threads - 1) / threads;
  d3q27_fp64_kernel<<<(unsigned)blocks, threads, 0, s>>>(a);
}

// Learned-alpha step with tensor-core inference: a persistent 128-thread
// block walks tiles of 128 consecutive nodes; per tile every thread gathers
// and prepares its node, the block runs the network on the tile with
// tcgen05.mma (mlp_tc_tile), and each thread finishes its node from the guess.
__global__ void __launch_bounds__(128, 2) d3q27_fp32_learned_tc_kernel(const Step27Args a) {
  extern __shared__ __align__(128) unsigned char smraw[];
  MlpTcSmem& s = *reinterpret_cast<MlpTcSmem*>(smraw);
  mlp_tc_setup(s, a.mlp);
  const float* __restrict__ src = static_cast<const float*>(a.src);
  const int64_t ntiles = (a.N + 127) / 128;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t n = tile * 128 + threadIdx.x;
    const uint8_t t = (n < a.N) ? __ldg(a.ntype + n) : (uint8_t)NT_SKIP;
    float d[Q];
    float2 D2[14], y2[14];
    float ymax = 0.f;
    bool bad = false;
    if (t != NT_SKIP) {
      gather(a, src, n, t, d);
      node_prepare(d, true, D2, y2, ymax, bad);
    }
    // features y / max|y| straight into the tile (zeros for a thread without a node)
    const float il = (t != NT_SKIP && ymax > 0.f) ? 1.0f / ymax : 0.f;
#pragma unroll
    for (int q = 0; q < 14; ++q) {
      const float v0 = (t != NT_SKIP) ? y2[q].x * il : 0.f;
      const float v1 = (t != NT_SKIP && 2 * q + 1 < Q) ? y2[q].y * il : 0.f;
      mlp_tc_put(s, 2 * q, v0, v1);
    }
    mlp_tc_put(s, 28, 0.f, 0.f);
    mlp_tc_put(s, 30, 0.f, 0.f);
    const float out = mlp_tc_run(s, &a.stats->status);
    if (t != NT_SKIP) node_finish<false, 1>(a, n, d, D2, y2, ymax, bad, ymax * out, ymax > 0.f ? 2 : -1);
  }
  mlp_tc_teardown(s);
}

// ---------------------------------------------------------------------------
// Negative-population repair (damp_it.f95:64-177, unshifted lattice).
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ double pop_f(const T* p, int64_t plane, int i, int64_t n);
template <>
__device__ __forceinline__ double pop_f<double>(const double* p, int64_t plane, int i, int64_t n) {
  return p[(int64_t)i * plane + n];
}
template <>
__device__ __forceinline__ double pop_f<float>(const float* p, int64_t plane, int i, int64_t n) {
  return (double)p[(int64_t)i * plane + n] + w27(i);
}

// Every fluid node's negative populations of the state a.src go to the list.
template <typename T>
__global__ void damp27_scan_kernel(const Step27Args a) {
  const T* __restrict__ f = static_cast<const T*>(a.src);
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < a.N; n += (int64_t)gridDim.x * blockDim.x) {
    if (__ldg(a.ntype + n) == NT_SKIP) continue;
    for (int i = 0; i < Q; ++i)
      if (pop_f(f, a.plane, i, n) < 0.0) {
        const unsigned long long slot = atomicAdd(a.neg_count, 1ull);
        if ((long long)slot < a.neg_cap) a.neg_list[slot] = (unsigned long long)n * Q + i;
      }
  }
}

// The repaired value of every listed population, from the unrepaired field.
// A link from x along c_i is a fluid link when the node pulls population
// opp(i) from x + c_i (and likewise for -c_i and population i).
template <typename T>
__global__ void damp27_value_kernel(const Step27Args a, T* __restrict__ vals) {
  const T* __restrict__ f = static_cast<const T*>(a.src);
  const long long cnt = (long long)min(*a.neg_count, (unsigned long long)a.neg_cap);
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x) {
    const unsigned long long idx = a.neg_list[e];
    const int64_t n = (int64_t)(idx / Q);
    const int i = (int)(idx % Q), o = opp27(i);
    int nx;
    int64_t nxy;
    box_strides(a, n, nx, nxy);
    const int64_t off = nbr_offset(i, nx, nxy);
    int64_t plus = -1, minus = -1;
    if (__ldg(a.ntype + n) == NT_BULK) {
      plus = n + off;
      minus = n - off;
    } else {
      const int32_t b = __ldg(a.bidx + n);
      const uint16_t wm = __ldg(a.words + (int64_t)b * Q + i), wp = __ldg(a.words + (int64_t)b * Q + o);
      if (lw_kind(wm) == LK_PULL && lw_pop(wm) == i && lw_off(wm) == off_code(-cx27(i), -cy27(i), -cz27(i)))
        minus = n - off;
      else if (lw_kind(wm) == LK_XBOX && lw_pop(wm) == i)
        minus = __ldg(a.xsrc + (int64_t)b * Q + i);
      if (lw_kind(wp) == LK_PULL && lw_pop(wp) == o && lw_off(wp) == off_code(cx27(i), cy27(i), cz27(i)))
        plus = n + off;
      else if (lw_kind(wp) == LK_XBOX && lw_pop(wp) == o)
        plus = __ldg(a.xsrc + (int64_t)b * Q + o);
    }
    const double v = pop_f(f, a.plane, i, n), av = fabs(v);
    double out = av;
    if (plus >= 0 && minus >= 0) {
      const double fp = pop_f(f, a.plane, i, plus), fm = pop_f(f, a.plane, i, minus);
      if (fp > 0.0 && fm > 0.0) out = (fp + fm) / 2.0;
      else if (fp > 0.0 && fm < 0.0) out = (fp + av) / 2.0;
      else if (fp < 0.0 && fm > 0.0) out = (fm + av) / 2.0;
    } else if (plus >= 0) {
      const double fp = pop_f(f, a.plane, i, plus);
      if (fp > 0.0) out = (fp + av) / 2.0;
    } else if (minus >= 0) {
      const double fm = pop_f(f, a.plane, i, minus);
      if (fm > 0.0) out = (fm + av) / 2.0;
    }
    vals[e] = (sizeof(T) == sizeof(float)) ? (T)(out - w27(i)) : (T)out;
  }
}

template <typename T>
__global__ void damp27_scatter_kernel(const Step27Args a, const T* __restrict__ vals) {
  T* __restrict__ f = static_cast<T*>(const_cast<void*>(a.src));
  const long long cnt = (long long)min(*a.neg_count, (unsigned long long)a.neg_cap);
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += (long long)gridDim.x * blockDim.x) {
    const unsigned long long idx = a.neg_list[e];
    f[(int64_t)(idx % Q) * a.plane + (int64_t)(idx / Q)] = vals[e];
  }
}

void launch_damp27_scan(const Step27Args& a, bool fp32, cudaStream_t s) {
  const unsigned grid = (unsigned)std::min<int64_t>((a.N + 255) / 256, 152 * 16);
  if (fp32) damp27_scan_kernel<float><<<grid, 256, 0, s>>>(a);
  else damp27_scan_kernel<double><<<grid, 256, 0, s>>>(a);
}

void launch_damp27_fix(const Step27Args& a, bool fp32, void* vals, cudaStream_t s) {
  if (fp32) {
    damp27_value_kernel<float><<<152 * 4, 256, 0, s>>>(a, static_cast<float*>(vals));
    damp27_scatter_kernel<float><<<152 * 4, 256, 0, s>>>(a, static_cast<const float*>(vals));
  } else {
    damp27_value_kernel<double><<<152 * 4, 256, 0, s>>>(a, static_cast<double*>(vals));
    damp27_scatter_kernel<double><<<152 * 4, 256, 0, s>>>(a, static_cast<const double*>(vals));
  }
}

bool staged_eligible(const Step27Args& a) {
  // one box; 16-byte aligned row segments: x rows and planes in multiples of 4 floats
  return a.nbox <= 1 && a.nx % 4 == 0 && a.plane % 4 == 0 && a.ny >= 3 && a.nz >= 3;
}

template <bool CHECK, int MODE>
void launch_staged(const Step27Args& a, cudaStream_t s) {
  static int blocks_per_sm = -1, sms = 0;
  const size_t smem = (size_t)kStages * kStageBytes;
  if (blocks_per_sm < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, d3q27_fp32_staged_kernel<CHECK, MODE>, 128, smem);
    if (blocks_per_sm < 1) blocks_per_sm = 1;
  }
  const int tiles_x = (a.nx + kTileX - 1) / kTileX;
  const int64_t ntiles = (int64_t)tiles_x * a.ny * a.nz;
  const int64_t grid = std::min<int64_t>(ntiles, (int64_t)sms * blocks_per_sm);
  d3q27_fp32_staged_kernel<CHECK, MODE><<<(unsigned)grid, 128, smem, s>>>(a);
}

// Returns whether the launched kernel updated every node (the learned-alpha
// tensor-core kernel); the other step kernels update the bulk nodes only.
bool launch_d3q27_fp32_main(const Step27Args& a, cudaStream_t s);

// Step kernel (bulk nodes), boundary kernel, then (with a list) the listed nodes.
void launch_d3q27_fp32(const Step27Args& a0, cudaStream_t s) {
  Step27Args a = a0;
  const bool defer = a.defer_list && a.alpha_mode == 1;  // Newton alpha (the learned guess keeps its own path)
  a.defer_on = defer ? 1 : 0;
  if (defer) cudaMemsetAsync(a.defer_count, 0, sizeof(unsigned long long), s);
  const bool all_nodes = launch_d3q27_fp32_main(a, s);
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  if (!all_nodes && a.nbnd > 0) {
    const long long bg = std::min<long long>((a.nbnd + 127) / 128, 1ll << 24);
    if (a.check_dH && a.alpha_mode == 2) d3q27_fp32_boundary_kernel<true, 1><<<(unsigned)bg, 128, 0, s>>>(a);
    else if (a.check_dH) d3q27_fp32_boundary_kernel<true, 0><<<(unsigned)bg, 128, 0, s>>>(a);
    else if (a.harvest) d3q27_fp32_boundary_kernel<false, 2><<<(unsigned)bg, 128, 0, s>>>(a);
    else if (a.alpha_mode == 2) d3q27_fp32_boundary_kernel<false, 1><<<(unsigned)bg, 128, 0, s>>>(a);
    else d3q27_fp32_boundary_kernel<false, 0><<<(unsigned)bg, 128, 0, s>>>(a);
  }
  if (!defer) return;
  const long long grid = std::min<long long>((a.defer_cap + 127) / 128, (long long)sms * 8);
  if (a.check_dH) d3q27_fp32_deferred_kernel<true, 0><<<(unsigned)grid, 128, 0, s>>>(a);
  else if (a.harvest) d3q27_fp32_deferred_kernel<false, 2><<<(unsigned)grid, 128, 0, s>>>(a);
  else d3q27_fp32_deferred_kernel<false, 0><<<(unsigned)grid, 128, 0, s>>>(a);
}

bool launch_d3q27_fp32_main(const Step27Args& a, cudaStream_t s) {
  const int threads = 128;
  const int64_t blocks = (a.N + threads - 1) / threads;
  if (a.alpha_mode == 2 && !a.check_dH && !a.harvest && a.mlp) {
    // learned alpha: tensor-core inference over 128-node tiles, persistent blocks
    static int bps = -1, sms = 0;
    if (bps < 0) {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, d3q27_fp32_learned_tc_kernel, 128, sizeof(MlpTcSmem));
      bps = bps < 1 ? 1 : (bps > 4 ? 4 : bps);  // at most 4 blocks x 128 TMEM columns per SM
    }
    const int64_t ntiles = (a.N + 127) / 128;
    const int64_t grid = std::min<int64_t>(ntiles, (int64_t)sms * bps);
    d3q27_fp32_learned_tc_kernel<<<(unsigned)grid, 128, sizeof(MlpTcSmem), s>>>(a);
    return true;
  }
  if (a.variant == kVariantTma && a.ws_maps && a.alpha_mode != 2 && !a.harvest) {
    static int bps = -1, sms = 0;
    const size_t smem = sizeof(WsSmem);
    if (bps < 0) {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaFuncSetAttribute(d3q27_fp32_ws_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      cudaFuncSetAttribute(d3q27_fp32_ws_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, d3q27_fp32_ws_kernel<false>, kWsThreads, smem);
      if (bps < 1) bps = 1;
    }
    const int64_t grid = std::min<int64_t>(a.ws_ntiles, (int64_t)sms * bps);
    if (a.check_dH) d3q27_fp32_ws_kernel<true><<<(unsigned)grid, kWsThreads, smem, s>>>(a);
    else d3q27_fp32_ws_kernel<false><<<(unsigned)grid, kWsThreads, smem, s>>>(a);
    return false;
  }
  if (a.variant == 3 && !a.check_dH && !a.harvest) {
    static int bps = -1, sms = 0;
    if (bps < 0) {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, d3q27_fp32_persistent_kernel<false, 4, 0>, 128, 0);
      if (bps < 1) bps = 1;
    }
    const int64_t grid = std::min<int64_t>(blocks, (int64_t)sms * bps);
    cudaMemsetAsync(a.work_counter, 0, sizeof(unsigned long long), s);
    if (a.alpha_mode == 2) d3q27_fp32_persistent_kernel<false, 4, 1><<<(unsigned)grid, threads, 0, s>>>(a);
    else d3q27_fp32_persistent_kernel<false, 4, 0><<<(unsigned)grid, threads, 0, s>>>(a);
    return false;
  }
  if (a.variant == 2 && !a.check_dH && !a.harvest && staged_eligible(a)) {
    if (a.alpha_mode == 2) launch_staged<false, 1>(a, s);
    else launch_staged<false, 0>(a, s);
    return false;
  }
  if (a.check_dH) {
    if (a.alpha_mode == 2) d3q27_fp32_kernel<true, 0, 1><<<(unsigned)blocks, threads, 0, s>>>(a);
    else d3q27_fp32_kernel<true, 0, 0><<<(unsigned)blocks, threads, 0, s>>>(a);
  } else if (a.harvest) {
    d3q27_fp32_kernel<false, 0, 2><<<(unsigned)blocks, threads, 0, s>>>(a);
  } else if (a.alpha_mode == 2) {
    if (a.variant == 1) d3q27_fp32_kernel<false, 4, 1><<<(unsigned)blocks, threads, 0, s>>>(a);
    else d3q27_fp32_kernel<false, 0, 1><<<(unsigned)blocks, threads, 0, s>>>(a);
  } else if (a.variant == 1) {
    d3q27_fp32_kernel<false, 4, 0><<<(unsigned)blocks, threads, 0, s>>>(a);
  } else if (a.variant == 4) {
    d3q27_fp32_kernel<false, 5, 0><<<(unsigned)blocks, threads, 0, s>>>(a);
  } else if (a.variant == 5) {
    d3q27_fp32_kernel<false, 6, 0><<<(unsigned)blocks, threads, 0, s>>>(a);
  } else if (a.variant == 6) {
    d3q27_fp32_kernel<false, 8, 0><<<(unsigned)blocks, threads, 0, s>>>(a);
  } else if (a.variant == 7) {
    d3q27_fp32_kernel<false, 7, 0><<<(unsigned)blocks, threads, 0, s>>>(a);
  } else if (a.variant == kVariantOff && a.pull_off_ok) {
    d3q27_fp32_kernel<false, 0, 0, true><<<(unsigned)blocks, threads, 0, s>>>(a);
  } else {
    d3q27_fp32_kernel<false, 0, 0><<<(unsigned)blocks, threads, 0, s>>>(a);
  }
  return false;
}

}  // namespace elbm
