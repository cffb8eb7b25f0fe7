/*
 * CPU FP64 oracle for the D3Q27 entropic lattice Boltzmann time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests, the smoke entry
 * point and the CPU-baseline leg of the benchmark load it; the product never
 * does.  It is a straight scalar restatement written for clarity, not speed.
 *
 * The reference solver has no working D3Q27 path (its D3Q27 velocity set is
 * declared in general/background_calcs/directions_and_weights.f95:236-244 but
 * no equilibrium or collision exists for it), so this oracle restates the
 * published entropic LBM (Ansumali, Karlin, Oettinger, EPL 63, 798, 2003:
 * D3Q27 entropic equilibrium, a product over the axes; Karlin, Ferrante,
 * Oettinger, EPL 47, 182, 1999: entropic alpha from H(f) = H(f + alpha*Delta))
 * on the reference's own D3Q27
 * ordering and link-code conventions:
 *   - directions, opposites: linking/modules/linkwise.f95:25-32 (cx_27 ... opp_27)
 *   - link codes in state(:,:,:,i): looping/timestepping/loop.f95:71-89 and the
 *     case ranges of looping/timestepping/streaming.f95:365-481
 *   - boundary rules: boundary_conditions/inlet_bc.f95:21-53, outlet_bc.f95:23-58,
 *     freestream_edge_bc.f95:18-19, pure_outflow_bc.f95:19-20,
 *     inviscid_edge.f95:25-1470 (specular reflection), bounceback.f95:13-19
 *   - step order streaming -> flow variables -> collision:
 *     looping/timestepping/loop.f95:94-147
 *
 * Streaming is written here in push form (like streaming.f95:266-1161) so the
 * GPU's pull form is checked against an independent formulation.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define Q 27

/* linkwise.f95:25-32 */
static const int CX[Q] = {0, 1, 0, 0, -1, 0, 0, 1, 0, -1, 0, 1, 1, -1, -1, 1, 0, -1, 0, 1, 1, 1, 1, -1, -1, -1, -1};
static const int CY[Q] = {0, 0, 1, 0, 0, -1, 0, 1, 1, 1, 1, 0, 0, 0, 0, -1, -1, -1, -1, 1, 1, -1, -1, 1, 1, -1, -1};
static const int CZ[Q] = {0, 0, 0, 1, 0, 0, -1, 0, -1, 0, 1, 1, -1, -1, 1, 0, -1, 0, 1, 1, -1, 1, -1, 1, -1, 1, -1};
static const int OPP[Q] = {0, 4, 5, 6, 1, 2, 3, 17, 18, 15, 16, 13, 14, 11, 12, 9, 10, 7, 8, 26, 25, 24, 23, 22, 21, 20, 19};

typedef struct {
  double nu;          /* kinematic viscosity, lattice units */
  double tol_alpha;   /* Newton step tolerance on alpha */
  int max_newton;     /* iteration cap */
  int alpha_mode;     /* 0: alpha = 2 (LBGK limit), 1: entropic Newton from alpha = 2 */
  double fs_feq[Q];   /* freestream equilibrium (codes -3, -8, -1000; outlet type 3) */
  double inl_feq[8][Q];
  double outl_feq[8][Q];
  int outlet_type[8]; /* 1,4: outlet equilibrium; 2: inlet table (press_temp_bc.f95:26-27); 3: freestream; 6: pure outflow */
} o27_params;

typedef struct {
  int64_t fluid_nodes;
  int64_t newton_iters;
  int64_t fallbacks;
  int64_t errors;
  double max_abs_dH;  /* max over nodes of |H(f + alpha Delta) - H(f)| */
} o27_stats;

static double weight(int i) {
  double w = 1.0;
  const int c[3] = {CX[i], CY[i], CZ[i]};
  for (int a = 0; a < 3; ++a) w *= (c[a] == 0) ? 2.0 / 3.0 : 1.0 / 6.0;
  return w;
}

/* Entropic equilibrium of D3Q27 (Ansumali, Karlin, Oettinger, Europhys. Lett. 63,
 * 798, 2003): the minimiser of H = sum f ln(f/w) at fixed rho and j, a product
 * over the axes of the D1Q3 solution
 *   f_i = rho * prod_a w1(c_ia) * psi(u_a) * zeta(u_a)^c_ia,
 *   psi(u) = 2 - sqrt(1 + 3u^2),  zeta(u) = (2u + sqrt(1 + 3u^2)) / (1 - u). */
void o27_equilibrium(double rho, const double u[3], double feq[Q]) {
  double g[3][3];
  for (int a = 0; a < 3; ++a) {
    const double s = sqrt(1.0 + 3.0 * u[a] * u[a]);
    const double psi = 2.0 - s;
    const double zeta = (2.0 * u[a] + s) / (1.0 - u[a]);
    g[a][1] = (2.0 / 3.0) * psi;
    g[a][2] = (1.0 / 6.0) * psi * zeta;
    g[a][0] = (1.0 / 6.0) * psi / zeta;
  }
  for (int i = 0; i < Q; ++i) feq[i] = rho * g[0][CX[i] + 1] * g[1][CY[i] + 1] * g[2][CZ[i] + 1];
}

void o27_weights(double w[Q]) {
  for (int i = 0; i < Q; ++i) w[i] = weight(i);
}

/* phi(x) = (1+x) ln(1+x) - x, with its Taylor series near 0 where the direct
 * form cancels. */
static double phi_fn(double x) {
  if (fabs(x) < 1e-2) {
    double p = 0.0;
    for (int n = 12; n >= 2; --n) p = p * (-x) + 1.0 / (n * (n - 1.0));
    return x * x * p;
  }
  return (1.0 + x) * log1p(x) - x;
}

/* Entropy difference H(f + alpha Delta) - H(f), H(f) = sum f ln(f/w), in the
 * form that holds when Delta conserves mass and momentum exactly:
 *   G(alpha) = sum_i f_i psi(y_i, alpha),  y_i = Delta_i / f_i,
 *   psi(y, a) = phi(a y) - a y ln(1 + y).
 * (Expanding (f + aD) ln((f + aD)/w) - f ln(f/w) = a D ln(f/w) + f (1+x) ln(1+x),
 * x = a y, and using ln(f/w) = ln(feq/w) - ln(1+y) with ln(feq/w) linear in
 * (1, c_i) for the entropic equilibrium, the terms a*sum D and a*sum c D vanish.)
 * Dropping those analytically-zero terms keeps the root insensitive to the
 * rounding residual of sum_i Delta_i, which the direct form multiplies by
 * alpha / H'(alpha) ~ 1/|Delta|^2. */
static double entropy_diff(const double* f, const double* d, const double* L1, double alpha) {
  double g = 0.0;
  for (int i = 0; i < Q; ++i) {
    const double y = d[i] / f[i];
    g += f[i] * (phi_fn(alpha * y) - alpha * y * L1[i]);
  }
  return g;
}

/* Entropic alpha by Newton from alpha = 2 on G(alpha) = 0 (non-trivial root),
 * safeguarded to the bracket (1, amax) of positive populations.  Returns alpha;
 * *iters = iterations; *fallback = 1 when the solve failed and alpha fell back
 * to 2 (clipped into the positivity bracket). */
double o27_alpha_newton(const double f[Q], const double d[Q], double tol, int max_it, int* iters, int* fallback) {
  double L1[Q];
  double s2 = 0.0, amax = INFINITY;
  for (int i = 0; i < Q; ++i) {
    L1[i] = log1p(d[i] / f[i]);
    s2 += d[i] * d[i] / f[i];
    if (d[i] < 0.0) {
      const double lim = -f[i] / d[i];
      if (lim < amax) amax = lim;
    }
  }
  *iters = 0;
  *fallback = 0;
  if (s2 < 1e-30) return 2.0;
  double alpha = (2.0 < amax) ? 2.0 : 0.5 * (1.0 + amax);
  int ok = 0;
  for (int it = 0; it < max_it; ++it) {
    double g = 0.0, gp = 0.0;
    for (int i = 0; i < Q; ++i) {
      const double y = d[i] / f[i];
      g += f[i] * (phi_fn(alpha * y) - alpha * y * L1[i]);
      gp += d[i] * (log1p(alpha * y) - L1[i]);
    }
    *iters = it + 1;
    if (!(gp > 0.0)) break;
    const double step = g / gp;
    double next = alpha - step;
    /* a Newton step that leaves the bracket (1, amax) is replaced by halving the way to its end */
    const int clipped = !(next > 1.0) || !(next < amax);
    if (!(next > 1.0)) next = 0.5 * (alpha + 1.0);
    else if (!(next < amax)) next = 0.5 * (alpha + amax);
    alpha = next;
    if (!clipped && fabs(step) <= tol) {
      ok = 1;
      break;
    }
  }
  if (!ok) {
    /* iteration cap with a small entropy residual still counts as converged */
    if (*iters >= max_it && fabs(entropy_diff(f, d, L1, alpha)) <= 1e-10) return alpha;
    *fallback = 1;
    return (2.0 < amax) ? 2.0 : 0.5 * (1.0 + amax);
  }
  return alpha;
}

double o27_entropy_diff(const double f[Q], const double d[Q], double alpha) {
  double L1[Q];
  for (int i = 0; i < Q; ++i) L1[i] = log1p(d[i] / f[i]);
  return entropy_diff(f, d, L1, alpha);
}

/* The direct form sum (f + alpha D) ln((f + alpha D)/w) - f ln(f/w), for reports. */
double o27_entropy_diff_direct(const double f[Q], const double d[Q], double alpha) {
  double w[Q], g = 0.0;
  o27_weights(w);
  for (int i = 0; i < Q; ++i) {
    const double x = alpha * d[i] / f[i];
    g += alpha * d[i] * log(f[i] / w[i]) + f[i] * (1.0 + x) * log1p(x);
  }
  return g;
}

/* Collision of one node: moments, equilibrium, alpha, f_out = f + alpha*beta*Delta. */
int o27_collide_node(const double f[Q], const o27_params* p, double fo[Q], double* alpha_out, int* iters,
                     int* fallback, double* dH) {
  double rho = 0.0, j[3] = {0, 0, 0};
  for (int i = 0; i < Q; ++i) {
    rho += f[i];
    j[0] += CX[i] * f[i];
    j[1] += CY[i] * f[i];
    j[2] += CZ[i] * f[i];
  }
  const double u[3] = {j[0] / rho, j[1] / rho, j[2] / rho};
  double feq[Q], d[Q];
  o27_equilibrium(rho, u, feq);
  for (int i = 0; i < Q; ++i) d[i] = feq[i] - f[i];
  double alpha = 2.0;
  *iters = 0;
  *fallback = 0;
  if (p->alpha_mode == 1) alpha = o27_alpha_newton(f, d, p->tol_alpha, p->max_newton, iters, fallback);
  *dH = (p->alpha_mode == 1) ? o27_entropy_diff(f, d, alpha) : 0.0;
  const double beta = 1.0 / (2.0 * p->nu / (1.0 / 3.0) + 1.0);
  for (int i = 0; i < Q; ++i) fo[i] = f[i] + alpha * beta * d[i];
  *alpha_out = alpha;
  return 0;
}

static inline int64_t idx(int x, int y, int z, int nx, int ny) { return ((int64_t)z * ny + y) * nx + x; }

static int node_is_fluid(int32_t s0) {
  /* collision.f95:157-159 skips state < 0, 1000 <= state < 51000, 200 <= state < 299 */
  if (s0 < 0) return 0;
  if (s0 >= 1000 && s0 < 51000) return 0;
  if (s0 >= 200 && s0 < 299) return 0;
  return 1;
}

/* One full time step on a single box without ghost cells:
 * fo_prev (post-collision of the previous step) -> push streaming with the
 * boundary rules -> moments, alpha, collision -> fo_next.
 * state: Q components of N int32 (component-major, x fastest), reference codes.
 * Returns 0, or a negative number for an unsupported link code / a fluid link
 * that leaves the box. */
int o27_step(int nx, int ny, int nz, const int32_t* state, const double* fo_prev, double* fo_next,
             const o27_params* p, double* alpha_out, int32_t* iters_out, o27_stats* st) {
  const int64_t N = (int64_t)nx * ny * nz;
  double* fi = (double*)malloc(sizeof(double) * Q * N);
  if (!fi) return -100;
  int rc = 0;
  /* fi starts as a copy of fo_prev so that links no rule writes keep a defined value */
  memcpy(fi, fo_prev, sizeof(double) * Q * N);
  memset(st, 0, sizeof(*st));
  for (int i = 0; i < Q && rc == 0; ++i) {
    for (int z = 0; z < nz && rc == 0; ++z)
      for (int y = 0; y < ny && rc == 0; ++y)
        for (int x = 0; x < nx; ++x) {
          const int64_t n = idx(x, y, z, nx, ny);
          if (!node_is_fluid(state[n])) continue;
          const int32_t code = (i == 0) ? 0 : state[(int64_t)i * N + n];
          const double fv = fo_prev[(int64_t)i * N + n];
          const int o = OPP[i];
          if (code >= 0) {
            const int xt = x + CX[i], yt = y + CY[i], zt = z + CZ[i];
            if (xt < 0 || yt < 0 || zt < 0 || xt >= nx || yt >= ny || zt >= nz) {
              rc = -2;
              break;
            }
            fi[(int64_t)i * N + idx(xt, yt, zt, nx, ny)] = fv;
          } else if (code == -10 || code == -5) {
            /* wall link: the population returns to its node reversed (halfway bounce-back) */
            fi[(int64_t)o * N + n] = fv;
          } else if (code == -11 || code == -12) {
            /* specular reflection: flip the components along every axis whose cardinal
             * link from this node is also an inviscid link, and drop those components
             * from the displacement (inviscid_edge.f95 case table) */
            int c[3] = {CX[i], CY[i], CZ[i]};
            int r[3] = {c[0], c[1], c[2]}, disp[3] = {c[0], c[1], c[2]};
            for (int a = 0; a < 3; ++a) {
              if (c[a] == 0) continue;
              int card = -1;
              for (int k = 1; k < 7; ++k) {
                const int ck[3] = {CX[k], CY[k], CZ[k]};
                if (ck[a] == c[a] && ck[(a + 1) % 3] == 0 && ck[(a + 2) % 3] == 0) card = k;
              }
              const int32_t cc = state[(int64_t)card * N + n];
              if (cc == -11 || cc == -12) {
                r[a] = -c[a];
                disp[a] = 0;
              }
            }
            int rd = -1;
            for (int k = 0; k < Q; ++k)
              if (CX[k] == r[0] && CY[k] == r[1] && CZ[k] == r[2]) rd = k;
            const int xt = x + disp[0], yt = y + disp[1], zt = z + disp[2];
            if (rd == i || xt < 0 || yt < 0 || zt < 0 || xt >= nx || yt >= ny || zt >= nz ||
                !node_is_fluid(state[idx(xt, yt, zt, nx, ny)])) {
              fi[(int64_t)o * N + n] = fv; /* no admissible mirror: reverse in place */
            } else {
              fi[(int64_t)rd * N + idx(xt, yt, zt, nx, ny)] = fv;
            }
          } else if (code == -3 || code == -8 || code == -1000) {
            fi[(int64_t)o * N + n] = p->fs_feq[o];
          } else if (code <= -100 && code >= -199) {
            const int k = -code - 100;
            if (k < 1 || k > 8) { rc = -3; break; }
            fi[(int64_t)o * N + n] = p->inl_feq[k - 1][o];
          } else if (code <= -200 && code >= -299) {
            const int k = -code - 200;
            if (k < 1 || k > 8) { rc = -3; break; }
            const int t = p->outlet_type[k - 1];
            double v;
            if (t == 1 || t == 4) v = p->outl_feq[k - 1][o];
            else if (t == 2) v = p->inl_feq[k - 1][o];
            else if (t == 3) v = p->fs_feq[o];
            else if (t == 6) v = fo_prev[(int64_t)o * N + n];
            else { rc = -4; break; }
            fi[(int64_t)o * N + n] = v;
          } else if (code == -666 || code == -1001) {
            /* null / solid neighbour without a wall fraction: nothing streams */
          } else if (code < -1001) {
            /* wall link with packed fraction (linkwise.f95:56), decoded as
             * interpolative_bounceback_bc.f95:66; linear interpolated bounce-back
             * (Bouzidi, Firdaouss, Lallemand 2001) */
            const double q = fabs((double)code + 1001.0) / 1e9;
            double v;
            const int xb = x - CX[i], yb = y - CY[i], zb = z - CZ[i];
            const int have2 = xb >= 0 && yb >= 0 && zb >= 0 && xb < nx && yb < ny && zb < nz &&
                              node_is_fluid(state[idx(xb, yb, zb, nx, ny)]);
            if (q < 0.5 && have2)
              v = 2.0 * q * fv + (1.0 - 2.0 * q) * fo_prev[(int64_t)i * N + idx(xb, yb, zb, nx, ny)];
            else if (q >= 0.5)
              v = fv / (2.0 * q) + (1.0 - 1.0 / (2.0 * q)) * fo_prev[(int64_t)o * N + n];
            else
              v = fv;
            fi[(int64_t)o * N + n] = v;
          } else {
            rc = -1;
            break;
          }
        }
  }
  if (rc == 0) {
    int64_t fluid = 0, newton = 0, fallbacks = 0;
    double maxdh = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : fluid, newton, fallbacks) reduction(max : maxdh)
    for (int64_t n = 0; n < N; ++n) {
      double f[Q], fo[Q];
      if (!node_is_fluid(state[n])) {
        for (int i = 0; i < Q; ++i) fo_next[(int64_t)i * N + n] = fo_prev[(int64_t)i * N + n];
        if (alpha_out) alpha_out[n] = 0.0;
        if (iters_out) iters_out[n] = 0;
        continue;
      }
      for (int i = 0; i < Q; ++i) f[i] = fi[(int64_t)i * N + n];
      double alpha, dH;
      int it, fb;
      o27_collide_node(f, p, fo, &alpha, &it, &fb, &dH);
      for (int i = 0; i < Q; ++i) fo_next[(int64_t)i * N + n] = fo[i];
      if (alpha_out) alpha_out[n] = alpha;
      if (iters_out) iters_out[n] = it;
      fluid++;
      newton += it;
      fallbacks += fb;
      if (fabs(dH) > maxdh) maxdh = fabs(dH);
    }
    st->fluid_nodes = fluid;
    st->newton_iters = newton;
    st->fallbacks = fallbacks;
    st->max_abs_dH = maxdh;
  }
  free(fi);
  return rc;
}

/* Macroscopic fields of a population array (rho, u) for error reports. */
void o27_moments(int64_t N, const double* f, double* rho, double* ux, double* uy, double* uz) {
  for (int64_t n = 0; n < N; ++n) {
    double r = 0, jx = 0, jy = 0, jz = 0;
    for (int i = 0; i < Q; ++i) {
      const double v = f[(int64_t)i * N + n];
      r += v;
      jx += CX[i] * v;
      jy += CY[i] * v;
      jz += CZ[i] * v;
    }
    rho[n] = r;
    ux[n] = jx / r;
    uy[n] = jy / r;
    uz[n] = jz / r;
  }
}

/* Solid nodes and wall-link fractions of a closed triangulated surface, by
 * testing every triangle for every node and link (the search of
 * lbgrid/inter_bb_setup.f95:44-246 and fluid_or_solid ray casting), in the
 * encoding of linkwise.f95:45-57.  Used to check the accelerated set-up code
 * bit for bit.  Node (i,j,k) sits at origin + (i,j,k) dx. */
static double o_seg_tri(const double* v, const double* p0, const double* p1) {
  const double a[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]}, b[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
  const double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
  const double dotv = n[0] * v[0] + n[1] * v[1] + n[2] * v[2];
  const double upper = dotv - (p0[0] * n[0] + p0[1] * n[1] + p0[2] * n[2]);
  const double lower = (p1[0] - p0[0]) * n[0] + (p1[1] - p0[1]) * n[1] + (p1[2] - p0[2]) * n[2];
  if (lower == 0.0) return -1.0;
  const double t = upper / lower;
  if (!(t > 0.0 && t <= 1.0)) return -1.0;
  const double xc[3] = {p0[0] + t * (p1[0] - p0[0]), p0[1] + t * (p1[1] - p0[1]), p0[2] + t * (p1[2] - p0[2])};
  double e[3][3];
  for (int k = 0; k < 3; ++k)
    for (int c = 0; c < 3; ++c) e[k][c] = v[3 * k + c] - p0[c];
  const double r[3] = {xc[0] - p0[0], xc[1] - p0[1], xc[2] - p0[2]};
#define VOL(A, B) (r[0] * (A[1] * B[2] - A[2] * B[1]) + r[1] * (A[2] * B[0] - A[0] * B[2]) + r[2] * (A[0] * B[1] - A[1] * B[0]))
  const double v1 = VOL(e[0], e[1]), v2 = -VOL(e[0], e[2]), v3 = VOL(e[1], e[2]);
#undef VOL
  const int pos = v1 >= 0.0 && v2 >= 0.0 && v3 >= 0.0, neg = v1 <= 0.0 && v2 <= 0.0 && v3 <= 0.0;
  return (pos || neg) ? t : -1.0;
}

static int o_ray_x(const double* v, const double* p) {
  const double y = p[1], z = p[2];
  const double y0 = v[1], z0 = v[2], y1 = v[4], z1 = v[5], y2 = v[7], z2 = v[8];
  const double det = (y1 - y0) * (z2 - z0) - (y2 - y0) * (z1 - z0);
  if (det == 0.0) return 0;
  double w[3];
  const double ay[3] = {y1, y2, y0}, az[3] = {z1, z2, z0}, by[3] = {y2, y0, y1}, bz[3] = {z2, z0, z1};
  for (int k = 0; k < 3; ++k) {
    double ww = (by[k] - ay[k]) * (z - az[k]) - (bz[k] - az[k]) * (y - ay[k]);
    if (ww == 0.0) ww = ((bz[k] > az[k]) || (bz[k] == az[k] && by[k] < ay[k])) ? 1e-300 : -1e-300;
    w[k] = (det < 0.0) ? -ww : ww;
  }
  if (!(w[0] > 0.0 && w[1] > 0.0 && w[2] > 0.0)) return 0;
  const double a[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]}, b[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
  const double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
  if (n[0] == 0.0) return 0;
  const double xs = v[0] - (n[1] * (y - y0) + n[2] * (z - z0)) / n[0];
  return xs > p[0];
}

#define RAY_DY 7.548776662466927e-7
#define RAY_DZ 5.698402909980532e-7

int o27_mark_triangles(int nx, int ny, int nz, const double* origin, double dx, int ntri, const double* tri,
                       int32_t* state) {
  const int64_t N = (int64_t)nx * ny * nz;
  char* solid = (char*)calloc(N, 1);
  if (!solid) return -1;
#pragma omp parallel for schedule(dynamic)
  for (int64_t n = 0; n < N; ++n) {
    const int i = (int)(n % nx), j = (int)((n / nx) % ny), k = (int)(n / ((int64_t)nx * ny));
    /* the ray starts a tiny irrational offset off the lattice line, so that it
     * passes through no vertex or edge of a surface built on lattice points */
    const double p[3] = {origin[0] + i * dx, origin[1] + (j + RAY_DY) * dx, origin[2] + (k + RAY_DZ) * dx};
    int cross = 0;
    for (int t = 0; t < ntri; ++t) cross += o_ray_x(tri + 9 * t, p);
    solid[n] = (char)(cross & 1);
  }
  for (int64_t n = 0; n < N; ++n)
    if (solid[n])
      for (int q = 0; q < Q; ++q) state[(int64_t)q * N + n] = -1001;
#pragma omp parallel for schedule(dynamic)
  for (int64_t n = 0; n < N; ++n) {
    if (solid[n]) continue;
    const int i = (int)(n % nx), j = (int)((n / nx) % ny), k = (int)(n / ((int64_t)nx * ny));
    const double p0[3] = {origin[0] + i * dx, origin[1] + j * dx, origin[2] + k * dx};
    for (int q = 1; q < Q; ++q) {
      /* only links from a fluid node to a solid node are wall links
       * (inter_bb_setup.f95:36-40: same-type neighbours skip the crossing search) */
      const int it = i + CX[q], jt = j + CY[q], kt = k + CZ[q];
      if (!(it >= 0 && jt >= 0 && kt >= 0 && it < nx && jt < ny && kt < nz && solid[idx(it, jt, kt, nx, ny)]))
        continue;
      const double p1[3] = {p0[0] + CX[q] * dx, p0[1] + CY[q] * dx, p0[2] + CZ[q] * dx};
      double tbest = INFINITY;
      for (int t = 0; t < ntri; ++t) {
        const double tt = o_seg_tri(tri + 9 * t, p0, p1);
        if (tt > 0.0 && tt < tbest) tbest = tt;
      }
      if (tbest == INFINITY) tbest = 1.0; /* the link ends in a solid node without a recorded crossing */
      const double len = sqrt((double)(CX[q] * CX[q] + CY[q] * CY[q] + CZ[q] * CZ[q])) * dx;
      const double dist = tbest * len;
      state[(int64_t)q * N + n] = -1001 - (int32_t)floor(dist / len * 1e9);
    }
  }
  free(solid);
  return 0;
}
