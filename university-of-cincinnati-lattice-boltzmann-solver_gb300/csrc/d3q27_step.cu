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

#include <cmath>
#include <cstdint>

#include "kernels.cuh"
#include "lattice.cuh"

namespace elbm {
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

// Gather the 27 streamed populations of node n (pull), bulk or boundary.
template <typename T>
__device__ __forceinline__ void gather(const Step27Args& a, const T* __restrict__ src, int64_t n, uint8_t t,
                                       T (&f)[Q]) {
  const int64_t nxy = (int64_t)a.nx * a.ny;
  if (t == NT_BULK) {
#pragma unroll
    for (int j = 0; j < Q; ++j) f[j] = load_src(src, a.plane, j, n - nbr_offset(j, a.nx, nxy));
  } else {
    const int32_t b = __ldg(a.bidx + n);
    const uint16_t* __restrict__ wp = a.words + (int64_t)b * Q;
    const T* __restrict__ eq = static_cast<const T*>(a.eq);
#pragma unroll
    for (int j = 0; j < Q; ++j) {
      const uint16_t w = __ldg(wp + j);
      const int kind = lw_kind(w);
      if (kind == LK_PULL) {
        const int off = lw_off(w);
        const int64_t s = n + (int64_t)(off % 3 - 1) + (int64_t)((off / 3) % 3 - 1) * a.nx +
                          (int64_t)(off / 9 - 1) * nxy;
        f[j] = load_src(src, a.plane, lw_pop(w), s);
      } else if (kind == LK_EQ) {
        f[j] = eq[lw_pop(w) * Q + j];
      } else {
        f[j] = load_src(src, a.plane, j, n);
      }
    }
  }
}

template <typename T>
__device__ __forceinline__ void store_dst(T* __restrict__ dst, int64_t plane, int64_t n, const T (&f)[Q]) {
#pragma unroll
  for (int j = 0; j < Q; ++j) dst[(int64_t)j * plane + n] = f[j];
}

__device__ __forceinline__ void warp_stats(DevStats* st, bool active, unsigned iters, bool exact, bool fb,
                                           unsigned flags, double dH) {
  const unsigned mask = __activemask();
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
    const unsigned long long m = ((unsigned long long)hi << 32) | lo;
    if (m) atomicMax(&st->max_dH_bits, m);
  }
}

// ---------------------------------------------------------------------------
// FP64 path: populations f_i in FP64, Newton on the exact entropy difference.
// Same algorithm and stopping rules as the CPU oracle.
// ---------------------------------------------------------------------------

__device__ double entropy_diff64(const double (&f)[Q], const double (&d)[Q], const double (&L)[Q], double alpha) {
  double g = 0.0;
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    const double x = alpha * d[i] / f[i];
    g += alpha * d[i] * L[i] + f[i] * (1.0 + x) * log1p(x);
  }
  return g;
}

__device__ double alpha_newton64(const double (&f)[Q], const double (&d)[Q], double tol, double tol_dH, int max_it,
                                 unsigned& iters, bool& fallback) {
  double L[Q];
  double s2 = 0.0, amax = INFINITY;
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    L[i] = log(f[i] / w27(i));
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
      const double x = alpha * d[i] / f[i];
      const double l1 = log1p(x);
      g += alpha * d[i] * L[i] + f[i] * (1.0 + x) * l1;
      gp += d[i] * (L[i] + l1 + 1.0);
    }
    iters = it + 1;
    if (!(gp > 0.0)) break;
    const double step = g / gp;
    const double next = alpha - step;
    if (!(next > 1.0) || !(next < amax)) break;
    alpha = next;
    if (fabs(step) <= tol) {
      ok = true;
      break;
    }
  }
  if (!ok) {
    if ((int)iters >= max_it && fabs(entropy_diff64(f, d, L, alpha)) <= tol_dH) return alpha;
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
      double Lg[Q];
#pragma unroll
      for (int i = 0; i < Q; ++i) Lg[i] = log(f[i] / w27(i));
      dH = fabs(entropy_diff64(f, d, Lg, alpha));
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
  store_dst(dst, a.plane, n, f);
  if (a.alpha_out) a.alpha_out[n] = (float)alpha;
  warp_stats(a.stats, true, iters, false, fb, flags, dH);
}

// ---------------------------------------------------------------------------
// FP32 path: deviations d_i = f_i - w_i stored in FP32; collision in FP32.
//
// Entropic alpha without cancellation: with y_i = Delta_i / f_i and the power
// sums S_n = sum_i f_i y_i^n, the entropy difference divided by alpha,
//   g(alpha) = [H(f + alpha Delta) - H(f)] / alpha,
// is  g(alpha) = A - sum_n (-1)^n S_n/(n-1) + sum_n (-1)^n S_n alpha^(n-1)/(n(n-1)),
// A = sum_i Delta_i ln(f^eq_i / w_i).  For the entropic equilibrium ln(f^eq/w)
// is linear in (1, c_i), so A = 0 by mass and momentum conservation.
// Expanded around alpha = 2 the S_2 terms cancel analytically, so
//   g(2 + delta) = sum_k t_k delta^k,  t_0 = sum_{n>=3} c_n S_n
// is evaluated from small quantities only; Newton runs on delta.  The series
// is used while max|y| <= kYSeries; beyond that the per-population logarithms
// are evaluated directly ("exact path").
// ---------------------------------------------------------------------------

constexpr int kNMax = 9;           // power sums S_2 .. S_9
constexpr float kYSeries = 0.06f;  // max |y| for the series path

__host__ __device__ constexpr double binom(int n, int k) {
  double r = 1.0;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}
__host__ __device__ constexpr double pow2i(int e) {
  double r = 1.0;
  for (int i = 0; i < e; ++i) r *= 2.0;
  return r;
}
__host__ __device__ constexpr double a_n(int n) { return ((n & 1) ? -1.0 : 1.0) / (n * (n - 1.0)); }
__host__ __device__ constexpr double b_n(int n) { return -((n & 1) ? -1.0 : 1.0) / (n - 1.0); }
// coefficient of S_n in t_0 and t_k
__host__ __device__ constexpr double c0(int n) { return a_n(n) * pow2i(n - 1) + b_n(n); }
__host__ __device__ constexpr double ck(int k, int n) { return (n - 1 >= k) ? a_n(n) * binom(n - 1, k) * pow2i(n - 1 - k) : 0.0; }

// phi(x) = (1+x) ln(1+x) - x and ln(1+x), accurate for all x > -1
__device__ __forceinline__ void phi_and_log1p(float x, float& phi, float& l1) {
  if (fabsf(x) < 0.125f) {
    // ln(1+x) = sum (-1)^(m+1) x^m / m ; phi(x) = sum_{n>=2} (-1)^n x^n/(n(n-1))
    float lp = 1.0f / 12.0f, pp = 1.0f / 132.0f;  // m = 12 ; n = 12
#pragma unroll
    for (int m = 11; m >= 1; --m) lp = fmaf(lp, -x, 1.0f / m);
    l1 = x * lp;
#pragma unroll
    for (int k = 11; k >= 2; --k) pp = fmaf(pp, -x, 1.0f / (k * (k - 1.0f)));
    phi = x * x * pp;
  } else {
    l1 = log1pf(x);
    phi = fmaf(1.0f + x, l1, -x);
  }
}

struct AlphaOut {
  float alpha;
  unsigned iters;
  bool exact;
  bool fallback;
};

// Direct FP32 Newton on G(alpha) = sum f psi(y, alpha),
// psi(y, a) = phi(a y) - a y ln(1+y), from alpha = 2 inside (1, amax).
__device__ AlphaOut alpha_exact32(const float (&fv)[Q], const float (&y)[Q], float amax, int max_it) {
  float Ly[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    float ph;
    phi_and_log1p(y[i], ph, Ly[i]);
  }
  float alpha = (2.0f < amax) ? 2.0f : 0.5f * (1.0f + amax);
  AlphaOut r{alpha, 0u, true, false};
  bool ok = false;
  for (int it = 0; it < max_it; ++it) {
    // G(a) = sum f [phi(a y) - a y Ly];  G'(a) = sum f y [ln(1+a y) - Ly]
    float G = 0.f, Gp = 0.f;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      float ph, l1;
      phi_and_log1p(alpha * y[i], ph, l1);
      const float fy = fv[i] * y[i];
      G += fv[i] * ph - alpha * fy * Ly[i];
      Gp += fy * (l1 - Ly[i]);
    }
    r.iters = it + 1;
    if (!(Gp > 0.0f)) break;
    const float step = G / Gp;
    const float next = alpha - step;
    if (!(next > 1.0f) || !(next < amax)) break;
    alpha = next;
    if (fabsf(step) <= 2e-7f * alpha) {
      ok = true;
      break;
    }
  }
  if (!ok) {
    r.fallback = true;
    alpha = (2.0f < amax) ? 2.0f : 0.5f * (1.0f + amax);
  }
  r.alpha = alpha;
  return r;
}

__global__ void __launch_bounds__(128) d3q27_fp32_kernel(const Step27Args a) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.N) return;
  const uint8_t t = __ldg(a.ntype + n);
  if (t == NT_SKIP) return;
  const float* __restrict__ src = static_cast<const float*>(a.src);
  float* __restrict__ dst = static_cast<float*>(a.dst);
  float d[Q];
  gather(a, src, n, t, d);

  // moments of the deviations: rho = 1 + sum d, j = sum c d (sum c w = 0)
  float dr = 0.f, jx = 0.f, jy = 0.f, jz = 0.f;
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    dr += d[i];
    if (cx27(i)) jx += cx27(i) * d[i];
    if (cy27(i)) jy += cy27(i) * d[i];
    if (cz27(i)) jz += cz27(i) * d[i];
  }
  const float rho = 1.0f + dr;
  const float inv_rho = 1.0f / rho;
  const float u[3] = {jx * inv_rho, jy * inv_rho, jz * inv_rho};
  // per-axis factor of the entropic equilibrium relative to its weight, minus one:
  // e_0 = psi - 1, e_+ = psi*zeta - 1, e_- = psi/zeta - 1, from small quantities only
  float e[3][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float uu = u[k] * u[k];
    const float sm1 = 3.0f * uu / (1.0f + sqrtf(fmaf(3.0f, uu, 1.0f)));  // sqrt(1+3u^2) - 1
    const float zm1 = (3.0f * u[k] + sm1) / (1.0f - u[k]);                 // zeta - 1
    e[k][1] = -sm1;
    e[k][2] = fmaf(1.0f - sm1, zm1, -sm1);
    e[k][0] = (-sm1 - zm1) / (1.0f + zm1);
  }
  // Delta_i = f^eq_i - f_i in deviation form: w_i [(1+P)(1+dr) - 1] - d_i, P = prod(1+e) - 1
  float D[Q];
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    const float A = e[0][cx27(i) + 1], B = e[1][cy27(i) + 1], C = e[2][cz27(i) + 1];
    const float P = fmaf(1.0f + A, fmaf(1.0f + B, C, B), A);
    const float wi = (float)w27(i);
    D[i] = fmaf(wi, fmaf(dr, 1.0f + P, P), -d[i]);
  }

  AlphaOut al{2.0f, 0u, false, false};
  double dH = 0.0;
  if (a.alpha_mode != 0) {
    float fv[Q], y[Q];
    float ymax = 0.f, amax = INFINITY;
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      fv[i] = (float)w27(i) + d[i];
      y[i] = __fdividef(D[i], fv[i]);
      ymax = fmaxf(ymax, fabsf(y[i]));
      if (y[i] < 0.f) amax = fminf(amax, -1.0f / y[i]);
    }
    if (ymax <= kYSeries) {
      float S[kNMax + 1];
#pragma unroll
      for (int k = 0; k <= kNMax; ++k) S[k] = 0.f;
#pragma unroll
      for (int i = 0; i < Q; ++i) {
        float p = D[i] * y[i];  // f y^2
        S[2] += p;
#pragma unroll
        for (int k = 3; k <= kNMax; ++k) {
          p *= y[i];
          S[k] += p;
        }
      }
      if (S[2] < 1e-30f) {
        al.alpha = 2.0f;
      } else {
        float tk[kNMax];  // t_0 .. t_{kNMax-1}
        tk[0] = 0.f;
#pragma unroll
        for (int nn = 3; nn <= kNMax; ++nn) tk[0] = fmaf((float)c0(nn), S[nn], tk[0]);
#pragma unroll
        for (int k = 1; k < kNMax; ++k) {
          float s = 0.f;
#pragma unroll
          for (int nn = 2; nn <= kNMax; ++nn)
            if (nn - 1 >= k) s = fmaf((float)ck(k, nn), S[nn], s);
          tk[k] = s;
        }
        float delta = 0.f;
        unsigned it = 0;
        bool ok = false;
        for (; it < 6;) {
          float p = tk[kNMax - 1], dp = 0.f;
#pragma unroll
          for (int k = kNMax - 2; k >= 0; --k) {
            dp = fmaf(dp, delta, p);
            p = fmaf(p, delta, tk[k]);
          }
          ++it;
          if (!(dp > 0.f)) break;
          const float step = p / dp;
          delta -= step;
          if (fabsf(step) <= 1e-7f * fmaxf(fabsf(delta), 1e-3f)) {
            ok = true;
            break;
          }
        }
        al.iters = it;
        const float alpha = 2.0f + delta;
        if (ok && alpha > 1.0f && alpha < amax) {
          al.alpha = alpha;
        } else {
          al = alpha_exact32(fv, y, amax, a.max_newton);
        }
      }
    } else {
      al = alpha_exact32(fv, y, amax, a.max_newton);
    }
    if (a.check_dH) {
      // |H(f + alpha Delta) - H(f)| in FP64 from the FP32 populations
      double g = 0.0;
      const double al64 = al.alpha;
#pragma unroll
      for (int i = 0; i < Q; ++i) {
        const double f64 = (double)w27(i) + (double)d[i];
        const double d64 = (double)D[i];
        const double x = al64 * d64 / f64;
        g += al64 * d64 * log(f64 / w27(i)) + f64 * (1.0 + x) * log1p(x);
      }
      dH = fabs(g);
    }
  }
  unsigned flags = 0;
  if (!isfinite(rho) || !isfinite(u[0]) || !isfinite(u[1]) || !isfinite(u[2])) flags |= 0x1u;
  if (al.fallback) flags |= 0x2u;
  if (a.check_dH && dH > a.tol_dH) flags |= 0x8u;
  const float ab = al.alpha * (float)a.beta;
  bool neg = false;
#pragma unroll
  for (int i = 0; i < Q; ++i) {
    d[i] = fmaf(ab, D[i], d[i]);
    neg |= (d[i] + (float)w27(i)) < 0.f;
  }
  if (neg) flags |= 0x4u;
  store_dst(dst, a.plane, n, d);
  if (a.alpha_out) a.alpha_out[n] = al.alpha;
  warp_stats(a.stats, true, al.iters, al.exact, al.fallback, flags, dH);
}

}  // namespace

void launch_d3q27_fp64(const Step27Args& a, cudaStream_t s) {
  const int threads = 128;
  const int64_t blocks = (a.N + threads - 1) / threads;
  d3q27_fp64_kernel<<<(unsigned)blocks, threads, 0, s>>>(a);
}

void launch_d3q27_fp32(const Step27Args& a, cudaStream_t s) {
  const int threads = 128;
  const int64_t blocks = (a.N + threads - 1) / threads;
  d3q27_fp32_kernel<<<(unsigned)blocks, threads, 0, s>>>(a);
}

}  // namespace elbm
