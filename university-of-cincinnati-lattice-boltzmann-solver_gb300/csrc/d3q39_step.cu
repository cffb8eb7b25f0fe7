// Fused D3Q39 compressible ELBM level step (two populations f, g; 13 Lagrange
// multipliers per node), FP64 arithmetic on FP64 or FP32-deviation storage,
// one thread per node.
//
// Replaces, for the reference's D3Q39 lattice, the per-level chain
//   streaming (looping/timestepping/streaming.f95:266-369, interior links)
//   calculate_flow_variables (calculate_flow_variables.f95:192-311)
//   collision (collision.f95:153-300)
// of looping/timestepping/loop.f95:104-139, with the same arithmetic:
//   moments, then the Newton solve of calculate_lagrangian_mults.f95:696-1097
//   with the Doolittle LU of lu_decomp.f95 (its two index quirks kept),
//   the closed-form alpha of calculate_alpha.f95:118-289, and the collision
//   with the heat-flux corrections of find_q_bar.f95 / find_little_q_bar.f95,
//   Sutherland viscosity and conductivity of quick_calcs.f95 and the
//   relaxation factors of amr_processes.f95:1751-1814.
// Streaming is pull-form over periodic images; the negative-population repair
// of damp_it.f95 runs as a second kernel.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <utility>

#include "kernels39.cuh"

// coefficient tables of the unshifted wall closure, in device memory
#define IBB39_QUAL __device__ const
#include "ibb39_table.h"

namespace elbm {

__constant__ Lattice39 c39;

// The integer tables as doubles (exact), so that the FP64 sums multiply by a
// constant operand instead of converting an integer in every term: the 13
// moment monomials, their 91 pairwise products (the Jacobian, r <= c row by
// row) and the third-moment tables of q-bar.
struct Lattice39D {
  double phi[13][39];
  double pp[91][39];
  double yi[27][39];
  double kr[27][39];
};
__constant__ Lattice39D c39d;

void upload_lattice39(const Lattice39& L, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(c39, &L, sizeof(L), 0, cudaMemcpyHostToDevice, s);
  static Lattice39D D;  // host staging (pageable: the copy completes before the call returns)
  int k = 0;
  for (int r = 0; r < 13; ++r) {
    for (int i = 0; i < 39; ++i) D.phi[r][i] = (double)L.phi[r][i];
    for (int c = r; c < 13; ++c, ++k)
      for (int i = 0; i < 39; ++i) D.pp[k][i] = (double)(L.phi[r][i] * L.phi[c][i]);
  }
  for (int m = 0; m < 27; ++m)
    for (int i = 0; i < 39; ++i) {
      D.yi[m][i] = (double)L.yi[m][i];
      D.kr[m][i] = (double)L.kroen[m][i];
    }
  cudaMemcpyToSymbolAsync(c39d, &D, sizeof(D), 0, cudaMemcpyHostToDevice, s);
}

namespace {

constexpr int Q = 39;
constexpr int NL = 13;

__device__ __forceinline__ double fieq39(double rho, const double (&lm)[NL], int i) {
  // amr_processes.f95:1729-1747, left-to-right sum of integer-weighted multipliers
  return rho * exp(lm[0] + c39d.phi[1][i] * lm[1] + c39d.phi[2][i] * lm[2] + c39d.phi[3][i] * lm[3] +
                   c39d.phi[4][i] * lm[4] + c39d.phi[5][i] * lm[5] + c39d.phi[6][i] * lm[6] +
                   c39d.phi[7][i] * lm[7] + c39d.phi[8][i] * lm[8] + c39d.phi[9][i] * lm[9] +
                   c39d.phi[10][i] * lm[10] + c39d.phi[11][i] * lm[11] + c39d.phi[12][i] * lm[12]);
}

// lu_decomp.f95: LU of J (row-major 13x13, overwritten), substitution,
// lm -= delta; returns max |delta|.
__device__ double lu_update39(double* J, const double (&target)[NL], double (&lm)[NL]) {
  // Doolittle in place: L (unit diagonal, below) and U (from the diagonal up) overwrite J row by
  // row; row 0 of U is row 0 of J, whose entries are also the moments the residual needs
  for (int r = 1; r < NL; ++r) {
    for (int c = 0; c < r; ++c) {
      double v = J[r * NL + c];
      for (int k = 0; k < c; ++k) {
        // lu_decomp.f95:105: lower(5,4) subtracts lower(5,2)*upper(3,4)
        const double l = (r == 4 && c == 3 && k == 2) ? J[4 * NL + 1] : J[r * NL + k];
        v -= l * J[k * NL + c];
      }
      J[r * NL + c] = (c == 0) ? J[r * NL] / J[0] : v / J[c * NL + c];
    }
    for (int c = r; c < NL; ++c) {
      double v = J[r * NL + c];
      for (int k = 0; k < r; ++k) v -= J[r * NL + k] * J[k * NL + c];
      J[r * NL + c] = v;
    }
  }
  double z[NL];
  for (int r = 0; r < NL; ++r) {
    double v = J[r] - target[r];
    for (int k = 0; k < r; ++k) {
      // lu_decomp.f95:441: z9 uses lower(9,7)*z8
      const double zz = (r == 8 && k == 6) ? z[7] : z[k];
      v -= J[r * NL + k] * zz;
    }
    z[r] = v;
  }
  double dl[NL];
  for (int r = NL - 1; r >= 0; --r) {
    double v = z[r];
    for (int c = NL - 1; c > r; --c) v -= J[r * NL + c] * dl[c];
    dl[r] = v / J[r * NL + r];
  }
  double md = fabs(dl[0]);
  for (int r = 1; r < NL; ++r) md = fabs(dl[r]) > md ? fabs(dl[r]) : md;
  for (int r = 0; r < NL; ++r) lm[r] -= dl[r];
  return md;
}

// The lattice tables at compile time for the two velocity sets the step runs
// most (LAT 1: unshifted; LAT 2: shifted along +x, primary flow direction 1;
// LAT 0: the tables in constant memory, any set).  With the integers known
// as template arguments, the zero terms of the Jacobian (53-62% of its 3,549
// products) and of the exponents drop out at compile time and the +-1 terms
// become additions: the same fused operations on the non-zero terms in the
// same order, so the same results, with about half the FP64 work of the
// multiplier Newton.
__host__ __device__ constexpr int cx39u(int i) {
  const int t[39] = {0, 1, 0, 0, -1, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 2, 0, 0, -2, 0,
                     0, 2, 2, 0, -2, -2, 2, 2, -2, -2, 0, 0, 0, 3, 0, 0, -3, 0, 0};
  return t[i];
}
__host__ __device__ constexpr int cy39u(int i) {
  const int t[39] = {0, 0, 1, 0, 0, -1, 0, 1, 1, -1, -1, 1, 1, -1, -1, 0, 2, 0, 0, -2,
                     0, 2, 0, 2, 2, -2, -2, 0, 0, 0, 2, -2, -2, 0, 3, 0, 0, -3, 0};
  return t[i];
}
__host__ __device__ constexpr int cz39u(int i) {
  const int t[39] = {0, 0, 0, 1, 0, 0, -1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 2, 0, 0,
                     -2, 0, 2, 2, 0, 0, 0, -2, -2, 2, -2, -2, 2, 0, 0, 3, 0, 0, -3};
  return t[i];
}
template <int LAT>
__host__ __device__ constexpr int phi39c(int r, int i) {
  const int x = cx39u(i) + (LAT == 2 ? 1 : 0), y = cy39u(i), z = cz39u(i);
  const int c2 = x * x + y * y + z * z;
  const int m[13] = {1, x, y, z, x * x, y * y, z * z, x * y, x * z, y * z, x * c2, y * c2, z * c2};
  return m[r];
}

// s += V * x as one fused operation, nothing for V = 0
template <int V>
__device__ __forceinline__ void fma39(double& s, double x) {
  if constexpr (V != 0) s = fma((double)V, x, s);
}

// the exponent of fieq39 for direction I: lm[0] + sum_r phi_r lm[r], left to right
template <int LAT, int I, int... R>
__device__ __forceinline__ double expo39(const double (&lm)[NL], std::integer_sequence<int, R...>) {
  double a = lm[0];
  (fma39<phi39c<LAT>(R + 1, I)>(a, lm[R + 1]), ...);
  return a;
}
template <int LAT, int... I>
__device__ __forceinline__ void fieq39_all(double rho, const double (&lm)[NL], double (&fe)[Q],
                                           std::integer_sequence<int, I...>) {
  ((fe[I] = rho * exp(expo39<LAT, I>(lm, std::make_integer_sequence<int, NL - 1>{}))), ...);
}

// Jacobian entry (R, C): sum_i phi_R phi_C fieq_i over the directions in order
template <int LAT, int R, int C, int... I>
__device__ __forceinline__ double jac39(const double (&fe)[Q], std::integer_sequence<int, I...>) {
  double s = 0.0;
  (fma39<phi39c<LAT>(R, I) * phi39c<LAT>(C, I)>(s, fe[I]), ...);
  return s;
}
template <int LAT, int R, int C>
__device__ __forceinline__ void jac39_cell(double* J, const double (&fe)[Q]) {
  if constexpr (C >= R) {
    const double s = jac39<LAT, R, C>(fe, std::make_integer_sequence<int, Q>{});
    J[R * NL + C] = s;
    J[C * NL + R] = s;
  }
}
template <int LAT, int R, int... C>
__device__ __forceinline__ void jac39_row(double* J, const double (&fe)[Q], std::integer_sequence<int, C...>) {
  (jac39_cell<LAT, R, C>(J, fe), ...);
}
template <int LAT, int... R>
__device__ __forceinline__ void jac39_all(double* J, const double (&fe)[Q], std::integer_sequence<int, R...>) {
  (jac39_row<LAT, R>(J, fe, std::make_integer_sequence<int, NL>{}), ...);
}

// The q-bar sums of direction I (find_q_bar.f95): sum over the 27 slots of
// m[qmap(slot)] times yi and kroen of the slot, in order, zero terms dropped.
__host__ __device__ constexpr int qmap39(int mm) {
  const int t[27] = {0, 3, 4, 3, 5, 6, 4, 6, 7, 3, 5, 6, 5, 1, 8, 6, 8, 9, 4, 6, 7, 6, 8, 9, 7, 9, 2};
  return t[mm];
}
template <int LAT>
__host__ __device__ constexpr int yi39c(int mm, int i) {
  const int x = cx39u(i) + (LAT == 2 ? 1 : 0), y = cy39u(i), z = cz39u(i);
  const int t[27] = {x * x * x, x * x * y, x * x * z, x * x * y, x * y * y, x * y * z, x * x * z, x * y * z, x * z * z,
                     x * x * y, x * y * y, x * y * z, x * y * y, y * y * y, y * y * z, x * y * z, y * y * z, z * z * y,
                     x * x * z, x * y * z, x * z * z, x * y * z, y * y * z, z * z * y, x * z * z, z * z * y, z * z * z};
  return t[mm];
}
template <int LAT>
__host__ __device__ constexpr int kr39c(int mm, int i) {
  const int x = cx39u(i) + (LAT == 2 ? 1 : 0), y = cy39u(i), z = cz39u(i);
  const int t[27] = {x, y, z, 0, 0, 0, 0, 0, 0, 0, 0, 0, x, y, z, 0, 0, 0, 0, 0, 0, 0, 0, 0, x, y, z};
  return t[mm];
}
template <int V>
__device__ __forceinline__ void fmaq39(double& s, double mv) {
  if constexpr (V != 0) s = fma(mv, (double)V, s);
}
template <int LAT, int I, int... M>
__device__ __forceinline__ void qbar39(const double (&m)[10], double& sy, double& sk, std::integer_sequence<int, M...>) {
  (fmaq39<yi39c<LAT>(M, I)>(sy, m[qmap39(M)]), ...);
  (fmaq39<kr39c<LAT>(M, I)>(sk, m[qmap39(M)]), ...);
}
// fn(std::integral_constant<int, i>) for every direction i, in order
template <class F, int... I>
__device__ __forceinline__ void each39(F&& fn, std::integer_sequence<int, I...>) {
  (fn(std::integral_constant<int, I>{}), ...);
}

// calculate_lagrangian_mults.f95:696-1097; returns iterations (negative at the cap).
template <int LAT = 0>
__device__ int lagrange39(int max_it, double rho, double u, double v, double w, double temp, const double (&P)[6],
                          double (&lm)[NL], double (&fieq)[Q]) {
  const double vel_mag = u * u + v * v + w * w;
  const double qx = (rho * vel_mag + 5 * rho * temp) * u;
  const double qy = (rho * vel_mag + 5 * rho * temp) * v;
  const double qz = (rho * vel_mag + 5 * rho * temp) * w;
  const double target[NL] = {rho, rho * u, rho * v, rho * w, P[0], P[1], P[2], P[3], P[4], P[5], qx, qy, qz};
  double max_diff = 1.0;
  int it = 0;
  double J[NL * NL];
  while (max_diff > 1.0e-7) {
    if (it >= max_it) return -it;
    ++it;
    if constexpr (LAT == 0) {
      for (int i = 0; i < Q; ++i) fieq[i] = fieq39(rho, lm, i);
      int k = 0;
      for (int r = 0; r < NL; ++r)
        for (int c = r; c < NL; ++c, ++k) {
          double s = 0.0;
          for (int i = 0; i < Q; ++i) s += c39d.pp[k][i] * fieq[i];
          J[r * NL + c] = s;
          J[c * NL + r] = s;
        }
    } else {
      fieq39_all<LAT>(rho, lm, fieq, std::make_integer_sequence<int, Q>{});
      jac39_all<LAT>(J, fieq, std::make_integer_sequence<int, NL>{});
    }
    max_diff = lu_update39(J, target, lm);
  }
  return it;
}

__device__ void sutherland39(const D3Q39Dev& k, double T, double& mu, double& dim_mu, double& dim_temp) {
  // quick_calcs.f95:24-64 (default-real literals rounded through float)
  const double const_s = (double)110.15f, temp_ref = (double)273.15f, visc_ref = 1.716e-5;
  const double unit_temp = T * k.t_ref * k.gama;
  const double unit_mu = visc_ref * pow(unit_temp / temp_ref, 1.5) * ((temp_ref + const_s) / (unit_temp + const_s));
  mu = unit_mu / k.mu_ref;
  dim_mu = unit_mu;
  dim_temp = unit_temp;
}

__device__ bool therm_cond39(const D3Q39Dev& k, double rho, double T, double& kappa) {
  // quick_calcs.f95:70-215, kappa_bottom = kappa_ref
  const double unit_temp = T * k.t_ref * k.gama;
  if (unit_temp <= 500.0) {
    kappa = 418.1 * (5.9776e-6 * pow(unit_temp, 1.5) / (unit_temp + (double)194.4f)) / k.kappa_ref;
    return true;
  }
  const double A[2][3][5] = {{{0.334316, 3.28202, 11.9939, 20.0944, 4.62882},
                              {0.413573, 3.83393, 13.1885, 20.7305, 4.27728},
                              {0.208749, 1.92122, 6.58813, 10.7630, -1.27699}},
                             {{10.9992, 387.106, 387.282, 5.48304, -1.20106},
                              {82.1184, 308.927, 423.174, 250.668, 47.5889},
                              {38.8677, 123.284, 144.224, 72.8083, 0.684807}}};
  double unit_p = unit_temp * (rho * k.rho_ref) * k.gas_const_R;
  int band;
  if (unit_temp <= 2250.0) {
    unit_p = (rho * k.rho_ref) * k.gas_const_R * unit_temp / 101300.0;
    band = 0;
  } else if (unit_temp <= 4250.0) {
    band = 1;
  } else {
    return false;
  }
  int row;
  if (unit_p < 10.0 && unit_p > 0.1) row = 0;
  else if (unit_p > 10.0 && unit_p < 100.0) row = 1;
  else if (unit_p > 100.0 && unit_p < 1000.0) row = 2;
  else return false;
  const double* c = A[band][row];
  const double kek = log(unit_temp / 10000.0);
  kappa = exp(c[0] * pow(kek, 4.0) + c[1] * pow(kek, 3.0) + c[2] * kek * kek + c[3] * kek + c[4]) / k.kappa_ref;
  return true;
}

__device__ __forceinline__ double eps39(const D3Q39Dev& k, int step) {
  // amr_processes.f95:1789-1814
  if (step < k.startup_timesteps) return ((double)step + 1.0) / (double)k.startup_timesteps * k.elbm_epsilon;
  return k.elbm_epsilon;
}

// calculate_alpha.f95:118-289
__device__ double alpha39(const D3Q39Dev& k, const double (&fi)[Q], const double (&fd)[Q], double temp, int step) {
  const double alpha_hi = 2.125, alpha_start = 1.0e-6, plus_epsilon = 1.24e-16, very_small = 1.0e-14;
  const double pi = 3.1415926535, k_boltz = 1.38064852e-23;
  double mu, dim_mu, dim_temp;
  sutherland39(k, temp, mu, dim_mu, dim_temp);
  const double mfp = dim_mu / k.p_ref * sqrt(pi * k_boltz * dim_temp / (2 * k.molec_weight));
  const double mft = mfp / sqrt(3 * k_boltz * dim_temp / k.molec_weight);
  const double bm = k.dt / (2 * mft + k.dt);
  double c1 = 0, c2 = 0, c3 = 0;
  for (int i = 0; i < Q; ++i) {
    const double df = fi[i] < 0.0 ? fabs(fi[i]) : fi[i];
    const double x = fd[i] / df;
    c1 = c1 + df * (2.0 * (x * x) / (2 + x));
    c2 = c2 + df * (x * x);
    if (x <= 0.0 && x >= -1.0) c3 = c3 + df * (x * x * x);
  }
  if (fabs(c3) < plus_epsilon) return 2.0;
  double asm_ = (c2 - sqrt(c2 * c2 - 8.0 * c3 * c1)) / (2.0 * c3);
  if (asm_ > alpha_hi) asm_ = alpha_hi - 1.0e-9;
  if (step < k.startup_timesteps) asm_ = (asm_ - alpha_start) / (double)k.startup_timesteps * step;
  double t1 = 0, t2 = 0, t3 = 0, t4 = 0, s1 = 0, s2 = 0, third = 0;
  for (int i = 0; i < Q; ++i) {
    const double df = fi[i] < 0.0 ? fabs(fi[i]) : fi[i];
    const double x1 = fd[i] / df, x2 = x1 * x1, x3 = x1 * x1 * x1;
    const double f2 = x2 * df, f3 = x3 * df, f4 = x2 * x2 * df, f5 = x2 * x3 * df, f6 = x3 * x3 * df;
    if (x1 <= 0.0 && x1 >= -1.0) {
      t1 = t1 + f3;
      t2 = t2 + f4;
      t3 = t3 + f5;
      t4 = t4 + f6;
    }
    s1 = s1 + f2;
    if (x1 >= 0.0) s2 = s2 + f3 * (2.0 / (4 + asm_ * x1) + 1.0 / (4 + 2 * asm_ * x1) + 2.0 / (4 + 3 * asm_ * x1));
    third = third - (60 * f2 + 60 * f3 + 11 * f4) / (60 + 90 * x1 + 36 * x2 + 3 * x3);
  }
  const double first = -(bm * bm) * (t1 / 6 - alpha_hi * bm * t2 / 12 + alpha_hi * alpha_hi * (bm * bm) * t3 / 20 -
                                     alpha_hi * alpha_hi * alpha_hi * (bm * bm * bm) * t4 / 5);
  const double second = s1 / 2 - 2 * asm_ * (bm * bm) * s2 / 15;
  if (fabs(first) < very_small) return 2.0;
  const double na = (-second + sqrt(second * second - 4 * first * third)) / (2 * first);
  if (na < asm_) return asm_;
  if (na > alpha_hi) return alpha_hi;
  return na;
}

// Population loads and stores of either storage: FP64 as is, FP32 as float
// deviations from the box's per-direction reference (ref[j] for f, ref[39 + j] for g).
template <bool F32>
__device__ __forceinline__ double ld_f39(const Step39Args& a, int pop, int64_t s) {
  if constexpr (F32) return (double)a.fsrc32[(int64_t)pop * a.plane + s] + a.ref[pop];
  else return a.fsrc[(int64_t)pop * a.plane + s];
}
template <bool F32>
__device__ __forceinline__ double ld_g39(const Step39Args& a, int pop, int64_t s) {
  if constexpr (F32) return (double)a.gsrc32[(int64_t)pop * a.plane + s] + a.ref[Q + pop];
  else return a.gsrc[(int64_t)pop * a.plane + s];
}
template <bool F32>
__device__ __forceinline__ void st_fg39(const Step39Args& a, int i, int64_t n, double f, double g) {
  if constexpr (F32) {
    a.fdst32[(int64_t)i * a.plane + n] = (float)(f - a.ref[i]);
    a.gdst32[(int64_t)i * a.plane + n] = (float)(g - a.ref[Q + i]);
  } else {
    a.fdst[(int64_t)i * a.plane + n] = f;
    a.gdst[(int64_t)i * a.plane + n] = g;
  }
}

template <bool F32, int LAT>
__global__ void __launch_bounds__(64) d3q39_step_kernel(const Step39Args a) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.N) return;
  const D3Q39Dev& k = a.k;
  const int x = (int)(n % a.nx), y = (int)((n / a.nx) % a.ny), z = (int)(n / ((int64_t)a.nx * a.ny));
  double f[Q], g[Q];
  const uint8_t t = a.ntype ? a.ntype[n] : (uint8_t)1;
  if (t == 0) return;  // neither pushes nor collides
  if (t == 1) {
    // pull streaming over periodic images: f_j(x) = fout_j(x - c_j)
    for (int j = 0; j < Q; ++j) {
      int sx = x - c39.cx[j], sy = y - c39.cy[j], sz = z - c39.cz[j];
      sx = (sx % a.nx + a.nx) % a.nx;
      sy = (sy % a.ny + a.ny) % a.ny;
      sz = (sz % a.nz + a.nz) % a.nz;
      const int64_t s = ((int64_t)sz * a.ny + sy) * a.nx + sx;
      f[j] = ld_f39<F32>(a, j, s);
      g[j] = ld_g39<F32>(a, j, s);
    }
  } else {
    // boundary record: what the push loop leaves in each post-streaming slot
    const int64_t b = a.bidx[n];
    for (int j = 0; j < Q; ++j) {
      const uint32_t w = a.words[b * Q + j];
      const uint32_t kind = w & 3u;
      const int pop = (int)((w >> 2) & 63u);
      if (kind == L39_PULL) {
        const int off = (int)(w >> 13);
        int sx = x + off % 9 - 4, sy = y + (off / 9) % 9 - 4, sz = z + off / 81 - 4;
        sx = (sx % a.nx + a.nx) % a.nx;
        sy = (sy % a.ny + a.ny) % a.ny;
        sz = (sz % a.nz + a.nz) % a.nz;
        const int64_t s = ((int64_t)sz * a.ny + sy) * a.nx + sx;
        f[j] = ld_f39<F32>(a, pop, s);
        g[j] = ld_g39<F32>(a, pop, s);
      } else if (kind == L39_EQ) {
        const int table = (int)((w >> 8) & 31u);
        f[j] = a.eqf[table * Q + pop];
        g[j] = a.eqg[table * Q + pop];
      } else if (kind == L39_WALL) {
        const int64_t r = a.recwall[b];
        f[j] = a.wallf[r * Q + pop];
        g[j] = a.wallg[r * Q + pop];
      } else {
        f[j] = a.fprev[b * Q + j];
        g[j] = a.gprev[b * Q + j];
      }
    }
    for (int j = 0; j < Q; ++j) {
      a.fprev[b * Q + j] = f[j];
      a.gprev[b * Q + j] = g[j];
    }
  }
  double lm[NL];
  for (int r = 0; r < NL; ++r) lm[r] = a.lm[(int64_t)r * a.plane + n];
  // calculate_flow_variables.f95:236-271: next to a wall the first steps solve from the start-up set
  if (t == 3 && k.shifted && a.step <= 1)
    for (int r = 0; r < NL; ++r) lm[r] = k.su_lm[r];
  // calculate_flow_variables.f95:201-228
  double rs = 0, us = 0, vs = 0, ws = 0, es = 0;
  for (int i = 0; i < Q; ++i) {
    rs = rs + f[i];
    us = us + c39.cx[i] * f[i];
    vs = vs + c39.cy[i] * f[i];
    es = es + c39.cmag[i] * f[i] + g[i];
  }
  const double rho = rs, u = us / rs, v = vs / rs;
  for (int i = 0; i < Q; ++i) ws = ws + c39.cz[i] * f[i];
  const double w = ws / rs;
  const double w_old = a.w_vel[n];
  const double vmag = u * u + v * v + w * w;
  const double temp = (es - rho * vmag) / (2 * k.const_vol * rho);
  const double P[6] = {rho * (temp + u * u), rho * (temp + v * v), rho * (temp + w_old * w_old),
                       rho * u * v,          rho * u * w,          rho * v * w};
  double fe[Q];
  int it = lagrange39<LAT>(k.max_lm_iters, rho, u, v, w, temp, P, lm, fe);
  unsigned flags = 0;
  if (it < 0) {
    flags |= 0x2u;
    it = -it;
    for (int i = 0; i < Q; ++i) fe[i] = fieq39(rho, lm, i);
  }
  double fd[Q];
  for (int i = 0; i < Q; ++i) fd[i] = fe[i] - f[i];
  const double alpha = k.turbulent ? alpha39(k, f, fd, temp, a.step) : 2.0;
  // collision.f95:153-300 with the final multipliers
  const double lead = 2.0 * k.const_vol - 3;
  double gd[Q];
  if constexpr (LAT != 0) fieq39_all<LAT>(rho, lm, fe, std::make_integer_sequence<int, Q>{});
  for (int i = 0; i < Q; ++i) {
    if constexpr (LAT == 0) fe[i] = fieq39(rho, lm, i);
    fd[i] = fe[i] - f[i];
    gd[i] = lead * temp * fe[i] - g[i];
  }
  const double eps = eps39(k, a.step);
  // find_q_bar.f95:33-220: ten central third moments of Delta f
  double m[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};  // xxx yyy zzz xxy xxz xyy xyz xzz yyz yzz
  for (int i = 0; i < Q; ++i) {
    const double X = c39.cx[i] - u, Y = c39.cy[i] - v, Z = c39.cz[i] - w;
    m[0] = m[0] + X * X * X * fd[i];
    m[1] = m[1] + Y * Y * Y * fd[i];
    m[2] = m[2] + Z * Z * Z * fd[i];
    m[3] = m[3] + (X * X) * Y * fd[i];
    m[4] = m[4] + (X * X) * Z * fd[i];
    m[5] = m[5] + (Y * Y) * X * fd[i];
    m[7] = m[7] + (Z * Z) * X * fd[i];
    m[8] = m[8] + (Y * Y) * Z * fd[i];
    m[9] = m[9] + (Z * Z) * Y * fd[i];
    m[6] = m[6] + X * Y * Z * fd[i];
  }
  // qabc(27) of find_q_bar.f95 as indices into m
  const int qmap[27] = {0, 3, 4, 3, 5, 6, 4, 6, 7, 3, 5, 6, 5, 1, 8, 6, 8, 9, 4, 6, 7, 6, 8, 9, 7, 9, 2};
  const double temp_coeff = 6.0 * (temp * temp * temp);
  // find_little_q_bar.f95:23-52
  double q1 = 0, q2 = 0, q3 = 0;
  for (int i = 0; i < Q; ++i) {
    q1 = q1 + (c39.cx[i] - u) * gd[i];
    q2 = q2 + (c39.cy[i] - v) * gd[i];
    q3 = q3 + (c39.cz[i] - w) * gd[i];
  }
  const double q_lead = eps / temp;
  double mu, dm, dt_;
  sutherland39(k, temp, mu, dm, dt_);
  double kappa = 0.0;
  if (!therm_cond39(k, rho, temp, kappa)) flags |= 0x10u;
  double b1, b2;
  if (a.step < k.startup_timesteps) {
    b1 = k.init_beta_1 + k.beta_1_scaling * a.step;
    b2 = k.init_beta_2 + k.beta_2_scaling * a.step;
  } else {
    b1 = 1.0 / ((pow(2.0, (double)(k.lvl + 1)) * mu) / (rho * temp) + 1.0);
    b2 = 1.0 / ((2.0 * kappa) / (rho * k.const_press * temp) + 1.0);
  }
  bool neg = false;
  if constexpr (LAT == 0) {
    for (int i = 0; i < Q; ++i) {
      double sy = 0.0, sk = 0.0;
      for (int mm = 0; mm < 27; ++mm) sy = sy + m[qmap[mm]] * c39d.yi[mm][i];
      for (int mm = 0; mm < 27; ++mm) sk = sk + m[qmap[mm]] * c39d.kr[mm][i];
      const double qb = eps * (sy - 3 * temp * sk) / temp_coeff;
      const double ch = q_lead * (c39.cx[i] * q1 + c39.cy[i] * q2 + c39.cz[i] * q3);
      const double fo = f[i] + alpha * b1 * (fd[i] - qb) + b2 * qb;
      const double go = g[i] + alpha * b1 * (gd[i] - ch) + b2 * ch;
      st_fg39<F32>(a, i, n, fo, go);
      neg |= fo < 0.0;
    }
  } else {
    (void)qmap;
    each39(
        [&](auto ic) {
          constexpr int i = decltype(ic)::value;
          double sy = 0.0, sk = 0.0;
          qbar39<LAT, i>(m, sy, sk, std::make_integer_sequence<int, 27>{});
          const double qb = eps * (sy - 3 * temp * sk) / temp_coeff;
          const double ch = q_lead * (c39.cx[i] * q1 + c39.cy[i] * q2 + c39.cz[i] * q3);
          const double fo = f[i] + alpha * b1 * (fd[i] - qb) + b2 * qb;
          const double go = g[i] + alpha * b1 * (gd[i] - ch) + b2 * ch;
          st_fg39<F32>(a, i, n, fo, go);
          neg |= fo < 0.0;
        },
        std::make_integer_sequence<int, Q>{});
  }
  for (int r = 0; r < NL; ++r) a.lm[(int64_t)r * a.plane + n] = lm[r];
  a.w_vel[n] = w;
  if (a.alpha) a.alpha[n] = alpha;
  if (a.macro) {
    a.macro[n] = rho;
    a.macro[a.plane + n] = u;
    a.macro[2 * a.plane + n] = v;
    a.macro[3 * a.plane + n] = w;
    a.macro[4 * a.plane + n] = temp;
  }
  if (!isfinite(rho) || !isfinite(temp)) flags |= 0x1u;
  if (neg) flags |= 0x4u;
  // per-warp aggregation of the counters
  const unsigned mask = __activemask();
  const unsigned sit = __reduce_add_sync(mask, (unsigned)it);
  const unsigned fl = __reduce_or_sync(mask, flags);
  const unsigned nn = __popc(mask);
  const unsigned capped = __popc(__ballot_sync(mask, (flags & 0x2u) != 0));
  if ((int)(threadIdx.x & 31) == __ffs(mask) - 1) {
    atomicAdd(&a.stats->node_updates, (unsigned long long)nn);
    atomicAdd(&a.stats->newton_iters, (unsigned long long)sit);
    if (capped) atomicAdd(&a.stats->fallbacks, (unsigned long long)capped);
    if (fl) atomicOr(&a.stats->status, fl);
  }
}

// ---- interpolated wall links on the shifted lattice ----

// derivatives.f95:816-1300: 1 when the derivative along axis (0 x, 1 y, 2 z)
// of direction i is the one-sided wall form (up: q_target - q_wall, else
// q_wall - q_target), 0 for the local difference.  Wall form on the axes where
// the unshifted velocity has a component, up when it is negative; the rest
// direction along x; directions 28, 30, 31 and 33 (1-based) carry the opposite
// up flags.
__device__ __forceinline__ bool wall_axis39(int i, int axis, bool& up) {
  const int c = axis == 0 ? c39.ucx[i] : axis == 1 ? c39.ucy[i] : c39.ucz[i];
  if (i == 0) {
    up = false;
    return axis == 0;
  }
  if (c == 0) return false;
  up = c < 0;
  if (i == 27 || i == 29 || i == 30 || i == 32) up = !up;
  return true;
}

// first_order_shifted_{vel,temp}_cond_unknown with dudx_ibb / dudx_local
__device__ double deriv39(double q_rest, double q_target, double q_up, double q_down, int i, int axis, int s_up,
                          int s_down, bool temperature) {
  bool up = false;
  if (wall_axis39(i, axis, up)) {
    const double dir_state = (fabs((double)s_down + 1001.0) / 1.0e9) * sqrt(c39.cmag[i]);
    const double q_wall = temperature ? q_target : 0.0;
    return up ? (q_target - q_wall) / (1.0 + dir_state) : (q_wall - q_target) / (1.0 + dir_state);
  }
  if (s_up >= 0 && s_down >= 0) return (q_down - q_up) / 2.0;
  if (s_up >= 0) return q_rest - q_up;
  if (s_down >= 0) return q_down - q_rest;
  return 0.0;
}

// shifted_ibb.f95:45-267 for wall link i: f and g of the missing population.
__device__ void shifted_ibb39(const D3Q39Dev& k, int i, int step, double fieq, double gieq, double rho, double ut,
                              double vt, double wt, double Tt, const double (&ul)[7], const double (&vl)[7],
                              const double (&wl)[7], const double (&Tl)[7], const int (&sp)[7], double& fout,
                              double& gout) {
  const double cv = k.const_vol;
  const double k_fi = -(rho * Tt) / 2.0;
  const double k_gi = -(rho * Tt * (2.0 * cv - 3)) / 2.0;
  const double eps = eps39(k, step);
  double mu, dm, dt_;
  sutherland39(k, Tt, mu, dm, dt_);
  double kappa = 0.0;
  therm_cond39(k, rho, Tt, kappa);
  double b1, b2;
  if (step < k.startup_timesteps) {
    b1 = k.init_beta_1 + k.beta_1_scaling * step;
    b2 = k.init_beta_2 + k.beta_2_scaling * step;
  } else {
    b1 = 1.0 / ((pow(2.0, (double)(k.lvl + 1)) * mu) / (rho * Tt) + 1.0);
    b2 = 1.0 / ((2.0 * kappa) / (rho * k.const_press * Tt) + 1.0);
  }
  double du[3], dv[3], dw[3], dT[3];
  for (int ax = 0; ax < 3; ++ax) {
    du[ax] = deriv39(ul[0], ut, ul[4 + ax], ul[1 + ax], i, ax, sp[4 + ax], sp[1 + ax], false);
    dv[ax] = deriv39(vl[0], vt, vl[4 + ax], vl[1 + ax], i, ax, sp[4 + ax], sp[1 + ax], false);
    dw[ax] = deriv39(wl[0], wt, wl[4 + ax], wl[1 + ax], i, ax, sp[4 + ax], sp[1 + ax], false);
    dT[ax] = deriv39(Tl[0], Tt, Tl[4 + ax], Tl[1 + ax], i, ax, sp[4 + ax], sp[1 + ax], true);
  }
  const double dudx = du[0], dudy = du[1], dudz = du[2], dvdx = dv[0], dvdy = dv[1], dvdz = dv[2];
  const double dwdx = dw[0], dwdy = dw[1], dwdz = dw[2], dTdx = dT[0], dTdy = dT[1], dTdz = dT[2];
  // 27 ordered pairs of the pressure-tensor gradient, then / beta_1
  const double sxy = dudy + dvdx, sxz = dudz + dwdx, syz = dvdz + dwdy;
  double p[27];
  p[0] = 2 * dudx - dudx / cv;
  p[1] = 2 * dudx - dvdy / cv;
  p[2] = 2 * dudx - dwdz / cv;
  p[3] = p[4] = p[5] = p[9] = p[10] = p[11] = sxy;
  p[6] = p[7] = p[8] = p[18] = p[19] = p[20] = sxz;
  p[12] = 2 * dvdy - dudx / cv;
  p[13] = 2 * dvdy - dvdy / cv;
  p[14] = 2 * dvdy - dwdz / cv;
  p[15] = p[16] = p[17] = p[21] = p[22] = p[23] = syz;
  p[24] = 2 * dwdz - dudx / cv;
  p[25] = 2 * dwdz - dvdy / cv;
  p[26] = 2 * dwdz - dwdz / cv;
  for (int m = 0; m < 27; ++m) p[m] = p[m] / b1;
  // third-moment gradients: ten distinct sums over the 27 slots
  const double qxxx = 3 * (dTdx / b2 + ut * p[0]);
  const double qxxy = (dTdy / b2 + vt * p[1] + 2 * ut * p[3]);
  const double qxxz = (dTdz / b2 + wt * p[2] + 2 * ut * p[6]);
  const double qxyx = (dTdy / b2 + 2 * ut * p[3] + vt * p[0]);
  const double qxyy = (dTdx / b2 + ut * p[12] + 2 * vt * p[3]);
  const double qxyz = (ut * p[21] + vt * p[6] + wt * p[3]);
  const double qxzz = (dTdx / b2 + ut * p[24] + 2 * wt * p[6]);
  const double qyxy = (dTdx / b2 + 2 * vt * p[3] + ut * p[12]);
  const double qyyy = 3 * (dTdy / b2 + vt * p[13]);
  const double qyyz = (dTdz / b2 + wt * p[14] + 2 * vt * p[21]);
  const double qyzz = (dTdy / b2 + vt * p[25] + 2 * wt * p[21]);
  const double qzxx = (dTdx / b2 + wt * p[2] + 2 * ut * p[6]);
  const double qzzz = 3 * (dTdz / b2 + wt * p[26]);
  const double q[27] = {qxxx, qxxy, qxxz, qxyx, qxyy, qxyz, qxxz, qxyz, qxzz, qxxy, qyxy, qxyz, qxyy, qyyy,
                        qyyz, qxyz, qyyz, qyzz, qzxx, qxyz, qxzz, qxyz, qyyz, qyzz, qxzz, qyzz, qzzz};
  const int cx = c39.cx[i], cy = c39.cy[i], cz = c39.cz[i];
  const double xx = cx * cx - Tt, yy = cy * cy - Tt, zz = cz * cz - Tt;
  // the reference's term order, its 25th pressure term counted twice
  const double p_comp =
      (p[0] * xx + p[1] * xx + p[2] * xx + p[3] * cx * cy + p[4] * cx * cy + p[5] * cx * cy + p[6] * cx * cz +
       p[7] * cx * cz + p[8] * cx * cz + p[9] * cy * cx + p[10] * cy * cx + p[11] * cy * cx + p[12] * yy +
       p[13] * yy + p[14] * yy + p[15] * cy * cz + p[16] * cy * cz + p[17] * cy * cz + p[18] * cz * cx +
       p[19] * cz * cx + p[20] * cz * cx + p[21] * cz * cy + p[22] * cz * cy + p[23] * cz * cy + p[24] * zz +
       p[24] * zz + p[25] * zz + p[26] * zz) /
      (2 * (Tt * Tt));
  const int cx2 = cx * cx, cy2 = cy * cy, cz2 = cz * cz;
  const double q_comp =
      (q[0] * (cx2 * cx - 3 * cx * Tt) + q[1] * (cx2 * cy - 3 * cy * Tt) + q[2] * (cx2 * cz - 3 * cz * Tt) +
       q[3] * cx2 * cy + q[4] * cx * cy2 + q[5] * cx * cy * cz + q[6] * cx2 * cz + q[7] * cx * cy * cz +
       q[8] * cx * cz2 + q[9] * cx2 * cy + q[10] * cy2 * cx + q[11] * cx * cy * cz +
       q[12] * (cy2 * cx - 3 * cx * Tt) + q[13] * (cy2 * cy - 3 * cy * Tt) + q[14] * (cy2 * cz - 3 * cz * Tt) +
       q[15] * cx * cy * cz + q[16] * cy2 * cz + q[17] * cz2 * cy + q[18] * cx2 * cz + q[19] * cx * cy * cz +
       q[20] * cz2 * cx + q[21] * cx * cy * cz + q[22] * cz * cy2 + q[23] * cz2 * cy +
       q[24] * (cz2 * cx - 3 * cx * Tt) + q[25] * (cz2 * cy - 3 * cy * Tt) + q[26] * (cz2 * cz - 3 * cz * Tt)) /
      (6 * (Tt * Tt * Tt));
  double fo = fieq + eps * k_fi * (p_comp + q_comp);
  const double k_one = 3 * (dTdx + dTdy + dTdz) / (b1 * cv);
  const double g_alpha = cx / Tt * (9 * dTdx / b2 + ut * k_one) + cy / Tt * (9 * dTdy / b2 + vt * k_one) +
                         cz / Tt * (9 * dTdz / b2 + wt * k_one);
  // heat-flux gradients of g (rab of shifted_ibb.f95), summed against c_a c_b - T delta_ab
  const double rxx0 = 2 * Tt * dudx + 2 * ut * dTdx - dudx / cv * (2 * Tt + ut * ut);
  const double rxx1 = 2 * Tt * dudx + 2 * ut * dTdx - dvdy / cv * (2 * Tt + ut * ut);
  const double rxx2 = 2 * Tt * dudx + 2 * ut * dTdx - dwdz / cv * (2 * Tt + ut * ut);
  const double rxy0 = Tt * (dudy + dvdx) + ut * dTdy + vt * dTdx - dudx / cv * ut * vt;
  const double rxy1 = Tt * (dudy + dvdx) + ut * dTdy + vt * dTdx - dvdy / cv * ut * vt;
  const double rxy2 = Tt * (dudy + dvdx) + ut * dTdy + vt * dTdx - dwdz / cv * ut * vt;
  const double rxz0 = Tt * (dudz + dwdx) + ut * dTdz + wt * dTdx - dudx / cv * ut * wt;
  const double rxz1 = Tt * (dudz + dwdx) + ut * dTdz + wt * dTdx - dvdy / cv * ut * wt;
  const double rxz2 = Tt * (dudz + dwdx) + ut * dTdz + wt * dTdx - dwdz / cv * ut * wt;
  const double ryy0 = 2 * Tt * dvdy + 2 * vt * dTdy - dudx / cv * (2 * Tt + vt * vt);
  const double ryy1 = 2 * Tt * dvdy + 2 * vt * dTdy - dvdy / cv * (2 * Tt + vt * vt);
  const double ryy2 = 2 * Tt * dvdy + 2 * vt * dTdy - dwdz / cv * (2 * Tt + vt * vt);
  const double ryz0 = Tt * (dvdz + dwdy) + wt * dTdy + vt * dTdz - dudx / cv * vt * wt;
  const double ryz1 = Tt * (dvdz + dwdy) + wt * dTdy + vt * dTdz - dvdy / cv * vt * wt;
  const double ryz2 = Tt * (dvdz + dwdy) + wt * dTdy + vt * dTdz - dwdz / cv * vt * wt;
  const double rzz0 = 2 * Tt * dwdz + 2 * wt * dTdz - dudx / cv * (2 * Tt + wt * wt);
  const double rzz1 = 2 * Tt * dwdz + 2 * wt * dTdz - dvdy / cv * (2 * Tt + wt * wt);
  const double rzz2 = 2 * Tt * dwdz + 2 * wt * dTdz - dwdz / cv * (2 * Tt + wt * wt);
  // rab(22..24) repeat rab(13..15) in the reference
  const double r_sum = rxx0 * xx + rxx1 * xx + rxx2 * xx + rxy0 * cx * cy + rxy1 * cx * cy + rxy2 * cx * cy +
                       rxz0 * cx * cz + rxz1 * cx * cz + rxz2 * cx * cz + rxy0 * cy * cx + rxy1 * cy * cx +
                       rxy2 * cy * cx + ryy0 * yy + ryy1 * yy + ryy2 * yy + ryz0 * cy * cz + ryz1 * cy * cz +
                       ryz2 * cy * cz + rxz0 * cz * cx + rxz1 * cz * cx + rxz2 * cz * cx + ryy0 * cz * cy +
                       ryy1 * cz * cy + ryy2 * cz * cy + rzz0 * zz + rzz1 * zz + rzz2 * zz;
  const double gi_neq = k_gi * (3 * k_one + g_alpha + r_sum / (2 * b1 * Tt));
  double go = gieq + eps * gi_neq;
  if (fo < 0.0) fo = fabs(fo);
  if (go < 0.0) go = fabs(go);
  fout = fo;
  gout = go;
}

// Sum of the closure terms [a, b) of one table: coefficient x derivative x u^. v^. w^. T^.
// beta_1^. beta_2^. C_v^., in table order.
__device__ double ibb39_poly(const ibb39_term* t, int a, int b, const double (&D)[12], double u, double v, double w,
                             double T, double b1, double b2, double cv) {
  const double iT = 1.0 / T, ib1 = 1.0 / b1, ib2 = 1.0 / b2, icv = 1.0 / cv;
  const double pu[4] = {1.0, u, u * u, u * u * u}, pv[4] = {1.0, v, v * v, v * v * v};
  const double pw[4] = {1.0, w, w * w, w * w * w};
  const double pT[8] = {iT * iT * iT * iT, iT * iT * iT, iT * iT, iT, 1.0, T, T * T, T * T * T};
  const double pb1[4] = {ib1 * ib1, ib1, 1.0, b1}, pb2[4] = {ib2 * ib2, ib2, 1.0, b2};
  const double pC[8] = {icv * icv, icv, 1.0, cv, cv * cv, cv * cv * cv, cv * cv * cv * cv, cv * cv * cv * cv * cv};
  double s = 0.0;
  for (int k = a; k < b; ++k) {
    const int e = t[k].e;
    s = s + t[k].c * D[e & 15] * pu[(e >> 4) & 3] * pv[(e >> 6) & 3] * pw[(e >> 8) & 3] * pT[(e >> 10) & 7] *
                pb1[(e >> 13) & 3] * pb2[(e >> 15) & 3] * pC[(e >> 17) & 7];
  }
  return s;
}

// interpolative_bounceback_bc.f95:834-2838 (unshifted lattice) for direction d = opp(i) of wall
// link i: dir_state from the node's own code of direction d; the one-sided wall derivatives
// (u_tgt - 0, T_tgt - T_tgt) over 1 + dir_state on the axes where c_d has a component (up when
// it is positive), the local differences on the others; the reference's hand-expanded
// non-equilibrium terms of direction d from the coefficient tables; no absolute value.
// Kept out of line: inlined into the wall kernel (255 registers) this build of the kernel
// returned NaN on the shifted path that never calls it; out of line both paths match the
// CPU restatement.
__device__ __noinline__ void unshifted_ibb39(const D3Q39Dev& k, int d, int code_d, int step, double fieq, double gieq,
                                double rho, double ut, double vt, double wt, double Tt, const double (&ul)[7],
                                const double (&vl)[7], const double (&wl)[7], const double (&Tl)[7],
                                const int (&sp)[7], double& fout, double& gout) {
  const double cv = k.const_vol;
  const double k_fi = -(rho * Tt) / 2.0;
  const double k_gi = -(rho * Tt * (2.0 * cv - 3)) / 2.0;
  const double eps = eps39(k, step);
  double mu, dm, dt_;
  sutherland39(k, Tt, mu, dm, dt_);
  double kappa = 0.0;
  therm_cond39(k, rho, Tt, kappa);
  double b1, b2;
  if (step < k.startup_timesteps) {
    b1 = k.init_beta_1 + k.beta_1_scaling * step;
    b2 = k.init_beta_2 + k.beta_2_scaling * step;
  } else {
    b1 = 1.0 / ((pow(2.0, (double)(k.lvl + 1)) * mu) / (rho * Tt) + 1.0);
    b2 = 1.0 / ((2.0 * kappa) / (rho * k.const_press * Tt) + 1.0);
  }
  const double dir_state = (fabs((double)code_d + 1001.0) / 1.0e9) * sqrt(c39.cmag[d]);
  const int c[3] = {c39.cx[d], c39.cy[d], c39.cz[d]};
  const double tgt[4] = {ut, vt, wt, Tt};
  double D[12];
  for (int q = 0; q < 4; ++q) {
    const double(&loc)[7] = q == 0 ? ul : q == 1 ? vl : q == 2 ? wl : Tl;
    for (int ax = 0; ax < 3; ++ax) {
      double v;
      if (c[ax] != 0) {
        const double q_wall = q == 3 ? tgt[3] : 0.0;
        v = c[ax] > 0 ? (tgt[q] - q_wall) / (1.0 + dir_state) : (q_wall - tgt[q]) / (1.0 + dir_state);
      } else {
        const int s_up = sp[4 + ax], s_down = sp[1 + ax];
        if (s_up >= 0 && s_down >= 0) v = (loc[1 + ax] - loc[4 + ax]) / 2.0;
        else if (s_up >= 0) v = loc[0] - loc[4 + ax];
        else if (s_down >= 0) v = loc[1 + ax] - loc[0];
        else v = 0.0;
      }
      D[3 * q + ax] = v;
    }
  }
  const double fn = k_fi * ibb39_poly(ibb39_f_terms, ibb39_f_off[d], ibb39_f_off[d + 1], D, ut, vt, wt, Tt, b1, b2, cv);
  const double gn = k_gi * ibb39_poly(ibb39_g_terms, ibb39_g_off[d], ibb39_g_off[d + 1], D, ut, vt, wt, Tt, b1, b2, cv);
  fout = fieq + eps * fn;
  gout = gieq + eps * gn;
}

// Value of a post-streaming slot described by a link word (PULL / EQ / STALE).
template <bool F32>
__device__ __forceinline__ void slot39(const Step39Args& a, uint32_t w, int64_t b, int j, int x, int y, int z,
                                       double& f, double& g) {
  const uint32_t kind = w & 3u;
  const int pop = (int)((w >> 2) & 63u);
  if (kind == L39_PULL) {
    const int off = (int)(w >> 13);
    int sx = x + off % 9 - 4, sy = y + (off / 9) % 9 - 4, sz = z + off / 81 - 4;
    sx = (sx % a.nx + a.nx) % a.nx;
    sy = (sy % a.ny + a.ny) % a.ny;
    sz = (sz % a.nz + a.nz) % a.nz;
    const int64_t s = ((int64_t)sz * a.ny + sy) * a.nx + sx;
    f = ld_f39<F32>(a, pop, s);
    g = ld_g39<F32>(a, pop, s);
  } else if (kind == L39_EQ) {
    const int table = (int)((w >> 8) & 31u);
    f = a.eqf[table * Q + pop];
    g = a.eqg[table * Q + pop];
  } else {
    f = a.fprev[b * Q + j];
    g = a.gprev[b * Q + j];
  }
}

// One thread per node with wall links: targets (target_finder.f95:36-58 on the
// unshifted lattice, :89-140 on the shifted one, and the Newton solve of
// streaming.f95:788-850, or the node's own previous fields when no wall link is
// among directions 1..14), the seven-point stencil (streaming.f95:577-603,
// 1055-1082) and, for every wall link, shifted_ibb or the unshifted closure.
// Reads the previous step's macroscopic planes, multipliers and post-collision
// populations before the step kernel overwrites them (same stream).
template <bool F32>
__global__ void __launch_bounds__(64) d3q39_wall_kernel(const Step39Args a) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= a.nwall) return;
  const D3Q39Dev& k = a.k;
  const Wall39Rec& R = a.walls[r];
  const int64_t n = R.node, b = R.rec;
  const int x = (int)(n % a.nx), y = (int)((n / a.nx) % a.ny), z = (int)(n / ((int64_t)a.nx * a.ny));
  const double* mrho = a.macro;
  const double* mu = a.macro + a.plane;
  const double* mv = a.macro + 2 * a.plane;
  const double* mT = a.macro + 4 * a.plane;
  const double* mw = a.w_vel;
  double rho_t, ut, vt, wt, Tt, lm[NL];
  unsigned flags = 0;
  int it = 0;
  if (R.adjacent) {
    int count = 0;
    double r_ = 0, u_ = 0, v_ = 0, w_ = 0, T_ = 0;
    for (int j = 0; j < Q; ++j) {
      const int32_t c = R.code[j];
      if (c <= -1001 && !k.shifted) {
        // target_finder.f95:36-58: the node across when that link is fluid, else the node itself
        const double d = fabs(((double)c + 1001.0) / 1.0e9);
        count++;
        const bool fluid = R.code[c39.opp[j]] >= 0;
        const int64_t m = fluid ? (int64_t)R.upass[c39.opp[j]] : n;
        u_ = u_ + (d * mu[m]) / (d + 1.0);
        v_ = v_ + (d * mv[m]) / (d + 1.0);
        w_ = w_ + (d * mw[m]) / (d + 1.0);
        T_ = T_ + (d * mT[m] + (fluid ? mT[m] : k.fs_temp)) / (d + 1.0);
      } else if (c <= -1001) {
        const double d = fabs(((double)c + 1001.0) / 1.0e9);
        count++;
        const int64_t m = R.upass[R.code[c39.erp[j]] == -666 ? j : 4];
        u_ = u_ + (d * mu[m]) / (d + 1.0);
        v_ = v_ + (d * mv[m]) / (d + 1.0);
        w_ = w_ + (d * mw[m]) / (d + 1.0);
        T_ = T_ + (d * mT[m] + mT[m]) / (d + 1.0);
      }
      const int s = R.code[c39.opp[j]] < -1000 ? c39.erp[j] : j;
      double fs, gs;
      slot39<F32>(a, R.snap[s], b, s, x, y, z, fs, gs);
      r_ = r_ + fs;
    }
    rho_t = r_;
    ut = u_ / count;
    vt = v_ / count;
    wt = w_ / count;
    Tt = T_ / count;
    for (int q = 0; q < NL; ++q) lm[q] = (k.shifted && a.step <= 4) ? k.su_lm[q] : a.lm[(int64_t)q * a.plane + n];
    const double P[6] = {rho_t * Tt + rho_t * (ut * ut), rho_t * Tt + rho_t * (vt * vt),
                         rho_t * Tt + rho_t * (wt * wt), rho_t * ut * vt, rho_t * ut * wt, rho_t * vt * wt};
    double fe[Q];
    it = lagrange39(k.max_lm_iters, rho_t, ut, vt, wt, Tt, P, lm, fe);
    if (it < 0) {
      flags |= 0x2u;
      it = -it;
    }
  } else {
    rho_t = mrho[n];
    ut = mu[n];
    vt = mv[n];
    wt = mw[n];
    Tt = mT[n];
    for (int q = 0; q < NL; ++q) lm[q] = a.lm[(int64_t)q * a.plane + n];
  }
  double ul[7], vl[7], wl[7], Tl[7];
  int sp[7];
  for (int j = 0; j < 7; ++j) {
    const int t = R.st[j];
    const int64_t m = R.sidx[j];
    sp[j] = t;
    if (t >= 0) {
      ul[j] = mu[m];
      vl[j] = mv[m];
      wl[j] = mw[m];
      Tl[j] = mT[R.adjacent ? m : (int64_t)R.tidx[j]];
    } else if (t == -11) {
      ul[j] = mu[n];
      vl[j] = mv[n];
      wl[j] = mw[n];
      Tl[j] = mT[n];
    } else if (t == -1000 || (t <= -100 && t >= -499)) {
      ul[j] = k.fs_u;
      vl[j] = k.fs_v;
      wl[j] = k.fs_w;
      Tl[j] = k.fs_temp;
    } else {
      ul[j] = 0.0;
      vl[j] = 0.0;
      wl[j] = 0.0;
      Tl[j] = k.fs_temp;
    }
  }
  for (int i = 1; i < Q; ++i) {
    if (R.code[i] > -1001) continue;
    // the equilibrium of direction opp(i) (= i on the shifted lattice)
    const int o = c39.opp[i];
    const double fieq = fieq39(rho_t, lm, o);
    const double gieq = (2.0 * k.const_vol - 3) * Tt * fieq;
    double fo, go;
    if (k.shifted)
      shifted_ibb39(k, i, a.step, fieq, gieq, rho_t, ut, vt, wt, Tt, ul, vl, wl, Tl, sp, fo, go);
    else
      unshifted_ibb39(k, o, R.code[o], a.step, fieq, gieq, rho_t, ut, vt, wt, Tt, ul, vl, wl, Tl, sp, fo, go);
    a.wallf[r * Q + i] = fo;
    a.wallg[r * Q + i] = go;
  }
  if (!isfinite(rho_t) || !isfinite(Tt)) flags |= 0x1u;
  if (it) atomicAdd(&a.stats->newton_iters, (unsigned long long)it);
  if (flags & 0x2u) atomicAdd(&a.stats->fallbacks, 1ull);
  if (flags) atomicOr(&a.stats->status, flags);
}

// Initial state of every node from its macroscopic fields
// (multilevel_initialization.f90:229-278 with the freestream multipliers of
// freestream_basis_calcs.f90:24-90 as the start): the multiplier Newton for
// rho, u, T and the equilibrium pressure tensor, then f = f_eq,
// g = (2 C_v - D) T f_eq, and the multipliers, w and the fields stored.
__global__ void __launch_bounds__(64) d3q39_init_kernel(const Step39Args a, const double* __restrict__ lm0,
                                                        unsigned long long* capped) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= a.N) return;
  const D3Q39Dev& k = a.k;
  const double rho = a.macro[n], u = a.macro[a.plane + n], v = a.macro[2 * a.plane + n],
               w = a.macro[3 * a.plane + n], T = a.macro[4 * a.plane + n];
  double lm[NL];
  for (int r = 0; r < NL; ++r) lm[r] = lm0[r];
  const double P[6] = {rho * (T + u * u), rho * (T + v * v), rho * (T + w * w), rho * u * v, rho * u * w, rho * v * w};
  double fe[Q];
  const int it = lagrange39(k.max_lm_iters, rho, u, v, w, T, P, lm, fe);
  if (it < 0) atomicAdd(capped, 1ull);
  const double lead = (2 * k.const_vol - 3) * T;
  for (int i = 0; i < Q; ++i) {
    const double f = fieq39(rho, lm, i);
    a.fdst[(int64_t)i * a.plane + n] = f;
    a.gdst[(int64_t)i * a.plane + n] = f * lead;
  }
  for (int r = 0; r < NL; ++r) a.lm[(int64_t)r * a.plane + n] = lm[r];
  a.w_vel[n] = w;
}

// Explosion into the fine ghost nodes of a D3Q39 level
// (interlevel_interpolation.f95:364-440), one thread per ghost node:
// f, g, the 13 multipliers, rho and T from the mean of the 1, 2, 4 or 8 coarse
// nodes around the node (nodal bilinear at ratio 2; src lists them z-, y-,
// x-major, sbox their coarse boxes); each population with f < 0, g < 0 or a
// NaN takes the coarse equilibrium f = f_eq(rho_c, lm_c), g = (2 C_v - D) T_c f;
// then the moments, the multiplier Newton from the interpolated multipliers
// and alpha of the node, as the reference does before the collision.
__global__ void __launch_bounds__(64) d3q39_explode_kernel(const Box39View* __restrict__ cb, const Box39View fb,
                                                           const int32_t* __restrict__ ghost,
                                                           const int32_t* __restrict__ src,
                                                           const uint16_t* __restrict__ sbox,
                                                           const uint8_t* __restrict__ cnt, int64_t n,
                                                           const D3Q39Dev k, int step,
                                                           unsigned long long* __restrict__ counters) {
  const int64_t gi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= n) return;
  const int kk = cnt[gi];
  const double inv = 1.0 / (double)kk;  // kk in {1, 2, 4, 8}: exact
  auto mean = [&](int which, int comp) {
    double s = 0.0;
    for (int m = 0; m < kk; ++m) {
      const Box39View& B = cb[sbox[8 * gi + m]];
      const double* p = which == 0 ? B.f : which == 1 ? B.g : which == 2 ? B.lm : B.macro;
      s += p[(int64_t)comp * B.plane + src[8 * gi + m]];
    }
    return s * inv;
  };
  double lmc[NL];
  for (int r = 0; r < NL; ++r) lmc[r] = mean(2, r);
  const double rho_c = mean(3, 0), temp_c = mean(3, 4);
  const double lead_c = (2 * k.const_vol - 3) * temp_c;
  double f[Q], g[Q];
  bool repaired = false;
  double rs = 0, us = 0, vs = 0, ws = 0, es = 0;
  for (int i = 0; i < Q; ++i) {
    f[i] = mean(0, i);
    g[i] = mean(1, i);
    if (!(f[i] >= 0.0) || !(g[i] >= 0.0)) {  // negative or NaN
      f[i] = fieq39(rho_c, lmc, i);
      g[i] = f[i] * lead_c;
      repaired = true;
    }
    rs = rs + f[i];
    us = us + c39.cx[i] * f[i];
    vs = vs + c39.cy[i] * f[i];
    ws = ws + c39.cz[i] * f[i];
    es = es + c39.cmag[i] * f[i] + g[i];
  }
  const double rho = rs, u = us / rs, v = vs / rs, w = ws / rs;
  const double vmag = u * u + v * v + w * w;
  const double temp = (es - rho * vmag) / (2 * k.const_vol * rho);
  const double P[6] = {rho * (temp + u * u), rho * (temp + v * v), rho * (temp + w * w),
                       rho * u * v,          rho * u * w,          rho * v * w};
  double lm[NL];
  for (int r = 0; r < NL; ++r) lm[r] = lmc[r];
  double fe[Q];
  const int it = lagrange39(k.max_lm_iters, rho, u, v, w, temp, P, lm, fe);
  if (it < 0)
    for (int i = 0; i < Q; ++i) fe[i] = fieq39(rho, lm, i);
  double alpha = 2.0;
  if (k.turbulent) {
    double fd[Q];
    for (int i = 0; i < Q; ++i) fd[i] = fe[i] - f[i];
    alpha = alpha39(k, f, fd, temp, step);
  }
  const int64_t d = ghost[gi];
  for (int i = 0; i < Q; ++i) {
    fb.f[(int64_t)i * fb.plane + d] = f[i];
    fb.g[(int64_t)i * fb.plane + d] = g[i];
  }
  for (int r = 0; r < NL; ++r) fb.lm[(int64_t)r * fb.plane + d] = lm[r];
  fb.w_vel[d] = w;
  fb.alpha[d] = alpha;
  const double mv[5] = {rho, u, v, w, temp};
  for (int r = 0; r < 5; ++r) fb.macro[(int64_t)r * fb.plane + d] = mv[r];
  if (repaired) atomicAdd(&counters[0], 1ull);
  if (it < 0) atomicAdd(&counters[1], 1ull);
}

// Coalescence onto a D3Q39 coarse box (fine_to_coarse.f95:13-45, nodal
// injection): coarse node dst[p] takes every per-node array of fine node
// src[p] of fine box sbox[p].  Thread e = component * n + p, so that a warp
// writes consecutive coarse entries of one plane.
constexpr int kDownComps39 = 2 * Q + NL + 1 + 1 + 5;  // f, g, lm, w, alpha, rho u v w T

__global__ void d3q39_average_down_kernel(const Box39View* __restrict__ fbs, const Box39View cbx,
                                          const int32_t* __restrict__ dst, const int32_t* __restrict__ src,
                                          const uint16_t* __restrict__ sbox, int64_t n) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * kDownComps39) return;
  const int c = (int)(e / n);
  const int64_t p = e - (int64_t)c * n;
  const Box39View& F = fbs[sbox[p]];
  const int64_t s = src[p], d = dst[p];
  const double* from;
  double* to;
  int comp;
  if (c < Q) {
    from = F.f, to = cbx.f, comp = c;
  } else if (c < 2 * Q) {
    from = F.g, to = cbx.g, comp = c - Q;
  } else if (c < 2 * Q + NL) {
    from = F.lm, to = cbx.lm, comp = c - 2 * Q;
  } else if (c == 2 * Q + NL) {
    from = F.w_vel, to = cbx.w_vel, comp = 0;
  } else if (c == 2 * Q + NL + 1) {
    from = F.alpha, to = cbx.alpha, comp = 0;
  } else {
    from = F.macro, to = cbx.macro, comp = c - (2 * Q + NL + 2);
  }
  to[(int64_t)comp * cbx.plane + d] = from[(int64_t)comp * F.plane + s];
}

}  // namespace

void launch_d3q39_fp64(const Step39Args& a, cudaStream_t s) {
  const int threads = 64;
  const int64_t blocks = (a.N + threads - 1) / threads;
  // the compile-time tables of the unshifted set and of the set shifted along +x
  const int lat = !a.k.shifted ? 1 : (a.k.primary_flow_dir == 1 ? 2 : 0);
  const unsigned g = (unsigned)blocks;
  if (a.fsrc32) {
    if (lat == 1) d3q39_step_kernel<true, 1><<<g, threads, 0, s>>>(a);
    else if (lat == 2) d3q39_step_kernel<true, 2><<<g, threads, 0, s>>>(a);
    else d3q39_step_kernel<true, 0><<<g, threads, 0, s>>>(a);
  } else {
    if (lat == 1) d3q39_step_kernel<false, 1><<<g, threads, 0, s>>>(a);
    else if (lat == 2) d3q39_step_kernel<false, 2><<<g, threads, 0, s>>>(a);
    else d3q39_step_kernel<false, 0><<<g, threads, 0, s>>>(a);
  }
}

// damp_it.f95:64-177 on one population set (fout, or gout: the reference
// applies the same rules to each) of a box with link codes (see the oracle's
// damp39_links for the rules).  dmask per node: bit i link i interior
// (unshifted: state >= 0; shifted: >= -500), bit 63 node type >= -500.
// Outside the box on a non-periodic axis a node type is -666 and the
// population the set's freestream equilibrium eq[i] (the initial value of the
// nodes outside an external-flow domain).  The reference repairs in place, direction by
// direction in z, y, x order, so a neighbour that comes earlier in that order
// and is itself negative is read repaired: damp39_value follows such chains
// (up to kDampChain links; longer chains read the unrepaired value).
// FP32 storage (src32 set): float deviations from ref, repaired values
// rounded back the same way and untouched ones copied as stored.
struct Damp39 {
  const double* src;
  const float* src32;
  const double* ref;
  const unsigned long long* dmask;
  const double* eq;
  int nx, ny, nz, periodic, shifted;
  int64_t plane;
  int3 lo, hi;
};
constexpr int kDampChain = 6;

__device__ int64_t damp39_node(const Damp39& P, int x, int y, int z) {
  if (P.periodic & 1) x = (x % P.nx + P.nx) % P.nx;
  else if (x < 0 || x >= P.nx) return -1;
  if (P.periodic & 2) y = (y % P.ny + P.ny) % P.ny;
  else if (y < 0 || y >= P.ny) return -1;
  if (P.periodic & 4) z = (z % P.nz + P.nz) % P.nz;
  else if (z < 0 || z >= P.nz) return -1;
  return ((int64_t)z * P.ny + y) * P.nx + x;
}

__device__ __forceinline__ double damp39_ld(const Damp39& P, int i, int64_t m) {
  return P.src32 ? (double)P.src32[(int64_t)i * P.plane + m] + P.ref[i] : P.src[(int64_t)i * P.plane + m];
}

__device__ double damp39_value(const Damp39& P, int i, int64_t n, int depth) {
  const double v = damp39_ld(P, i, n);
  if (!(v < 0.0)) return v;
  const int x = (int)(n % P.nx), y = (int)((n / P.nx) % P.ny), z = (int)(n / ((int64_t)P.nx * P.ny));
  const int cx = c39.cx[i], cy = c39.cy[i], cz = c39.cz[i];
  const int64_t mp = damp39_node(P, x + cx, y + cy, z + cz), mm = damp39_node(P, x - cx, y - cy, z - cz);
  auto read = [&](int64_t m) -> double {
    if (m < 0) return P.eq[i];
    if (m < n && depth > 0) return damp39_value(P, i, m, depth - 1);  // already repaired in the sweep
    return damp39_ld(P, i, m);
  };
  const double fp = read(mp), fm = read(mm);
  const unsigned long long msk = P.dmask ? P.dmask[n] : ~0ull;  // no link codes: every link interior
  const bool si = (msk >> i) & 1ull;
  bool four = false, plus = false, minus = false;
  double out = v;
  if (!P.shifted) {
    const bool so = (msk >> c39.opp[i]) & 1ull;
    four = si && so;
    plus = si && !so;
    minus = !si && so;
    if (!four && !plus && !minus) out = fabs(v);
  } else {
    const int a = P.lo.x + x, b = P.lo.y + y, c = P.lo.z + z, ngm = 8;
    const bool edge = a - cx < P.lo.x - ngm || a - cx < P.lo.y - ngm || c - cz < P.lo.z - ngm ||
                      a + cx > P.hi.x - ngm || b + cy > P.hi.y - ngm || c + cz > P.hi.z - ngm;
    if (edge) {
      out = si ? (fp + fabs(v)) / 2 : fabs(v);
    } else {
      const bool up = mm >= 0 && (!P.dmask || ((P.dmask[mm] >> 63) & 1ull));
      four = si && up;
      plus = si && !up;
      minus = !si && up;
    }
  }
  if (four) {
    if (fp > 0.0 && fm > 0.0) out = (fp + fm) / 2.0;
    else if (fp > 0.0 && fm < 0.0) out = (fp + fabs(v)) / 2;
    else if (fp < 0.0 && fm > 0.0) out = (fm + fabs(v)) / 2;
    else out = fabs(v);
  } else if (plus) {
    out = fp > 0.0 ? (fp + fabs(v)) / 2 : fabs(v);
  } else if (minus) {
    out = fm > 0.0 ? (fm + fabs(v)) / 2 : fabs(v);
  }
  return out;
}

__global__ void d3q39_damp_links_kernel(const Damp39 P, void* __restrict__ dst, DevStats* stats) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (n >= (int64_t)P.nx * P.ny * P.nz) return;
  const int64_t e = (int64_t)i * P.plane + n;
  const double v = damp39_ld(P, i, n);
  if (v < 0.0) {
    const double out = damp39_value(P, i, n, kDampChain);
    atomicAdd(&stats->exact_nodes, 1ull);
    if (P.src32) static_cast<float*>(dst)[e] = (float)(out - P.ref[i]);
    else static_cast<double*>(dst)[e] = out;
  } else if (P.src32) {
    static_cast<float*>(dst)[e] = P.src32[e];
  } else {
    static_cast<double*>(dst)[e] = P.src[e];
  }
}

void launch_d3q39_damp_links(const void* src, void* dst, const double* ref, const unsigned long long* dmask, int nx,
                             int ny, int nz, int64_t plane, int periodic, int shifted, const int* lo, const int* hi,
                             const double* eq, DevStats* stats, cudaStream_t s) {
  const int64_t N = (int64_t)nx * ny * nz;
  Damp39 P{ref ? nullptr : static_cast<const double*>(src), ref ? static_cast<const float*>(src) : nullptr, ref,
           dmask, eq, nx, ny, nz, periodic, shifted, plane, make_int3(lo[0], lo[1], lo[2]),
           make_int3(hi[0], hi[1], hi[2])};
  dim3 grid((unsigned)((N + 255) / 256), 39);
  d3q39_damp_links_kernel<<<grid, 256, 0, s>>>(P, dst, stats);
}

void launch_d3q39_init(const Step39Args& a, const double* lm0, unsigned long long* capped, cudaStream_t s) {
  const int threads = 64;
  d3q39_init_kernel<<<(unsigned)((a.N + threads - 1) / threads), threads, 0, s>>>(a, lm0, capped);
}

void launch_d3q39_walls(const Step39Args& a, cudaStream_t s) {
  if (a.nwall <= 0) return;
  const int threads = 64;
  const unsigned blocks = (unsigned)((a.nwall + threads - 1) / threads);
  if (a.fsrc32) d3q39_wall_kernel<true><<<blocks, threads, 0, s>>>(a);
  else d3q39_wall_kernel<false><<<blocks, threads, 0, s>>>(a);
}

void launch_d3q39_explode(const Box39View* coarse, const Box39View& fine, const int32_t* ghost, const int32_t* src,
                          const uint16_t* sbox, const uint8_t* cnt, int64_t n, const D3Q39Dev& k, int step,
                          unsigned long long* counters, cudaStream_t s) {
  if (n <= 0) return;
  const int threads = 64;
  d3q39_explode_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, s>>>(coarse, fine, ghost, src, sbox,
                                                                                   cnt, n, k, step, counters);
}

void launch_d3q39_average_down(const Box39View* fine, const Box39View& coarse, const int32_t* dst, const int32_t* src,
                               const uint16_t* sbox, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  const int64_t total = n * kDownComps39;
  d3q39_average_down_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(fine, coarse, dst, src, sbox, n);
}


}  // namespace elbm

namespace elbm {

// Host-side tables (directions_and_weights.f95:463-780).
void build_lattice39(int shifted, int primary_flow_dir, Lattice39& L) {
  static const int CX0[39] = {0, 1, 0, 0, -1, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 2, 0, 0, -2, 0,
                              0, 2, 2, 0, -2, -2, 2, 2, -2, -2, 0, 0, 0, 3, 0, 0, -3, 0, 0};
  static const int CY0[39] = {0, 0, 1, 0, 0, -1, 0, 1, 1, -1, -1, 1, 1, -1, -1, 0, 2, 0, 0, -2,
                              0, 2, 0, 2, 2, -2, -2, 0, 0, 0, 2, -2, -2, 0, 3, 0, 0, -3, 0};
  static const int CZ0[39] = {0, 0, 0, 1, 0, 0, -1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 2, 0, 0,
                              -2, 0, 2, 2, 0, 0, 0, -2, -2, 2, -2, -2, 2, 0, 0, 3, 0, 0, -3};
  static const int OPP0[39] = {1, 5, 6, 7, 2, 3, 4, 14, 15, 12, 13, 10, 11, 8, 9, 19, 20, 21, 16, 17,
                               18, 26, 29, 32, 27, 22, 25, 30, 23, 28, 33, 24, 31, 37, 38, 39, 34, 35, 36};
  for (int i = 0; i < 39; ++i) {
    int x = CX0[i], y = CY0[i], z = CZ0[i];
    if (shifted) {
      if (primary_flow_dir == 1) x += 1;
      else if (primary_flow_dir == 2) y += 1;
      else if (primary_flow_dir == 3) z += 1;
      else if (primary_flow_dir == 4) x -= 1;
      else if (primary_flow_dir == 5) y -= 1;
      else if (primary_flow_dir == 6) z -= 1;
    }
    L.cx[i] = x;
    L.cy[i] = y;
    L.cz[i] = z;
    L.opp[i] = shifted ? i : OPP0[i] - 1;
    L.ucx[i] = CX0[i];
    L.ucy[i] = CY0[i];
    L.ucz[i] = CZ0[i];
    L.erp[i] = OPP0[i] - 1;
    L.cmag[i] = (double)x * x + (double)y * y + (double)z * z;
    const int c2 = x * x + y * y + z * z;
    const int mono[13] = {1, x, y, z, x * x, y * y, z * z, x * y, x * z, y * z, x * c2, y * c2, z * c2};
    for (int r = 0; r < 13; ++r) L.phi[r][i] = mono[r];
    const int cxxx = x * x * x, cyyy = y * y * y, czzz = z * z * z, cxyz = x * y * z;
    const int cxxy = x * x * y, cxyy = x * y * y, cxxz = x * x * z, cxzz = x * z * z, cyyz = y * y * z,
              cyzz = z * z * y;
    const int yi[27] = {cxxx, cxxy, cxxz, cxxy, cxyy, cxyz, cxxz, cxyz, cxzz, cxxy, cxyy, cxyz, cxyy, cyyy,
                        cyyz, cxyz, cyyz, cyzz, cxxz, cxyz, cxzz, cxyz, cyyz, cyzz, cxzz, cyzz, czzz};
    const int kr[27] = {x, y, z, 0, 0, 0, 0, 0, 0, 0, 0, 0, x, y, z, 0, 0, 0, 0, 0, 0, 0, 0, 0, x, y, z};
    for (int m = 0; m < 27; ++m) {
      L.yi[m][i] = yi[m];
      L.kroen[m][i] = kr[m];
    }
  }
}

}  // namespace elbm
