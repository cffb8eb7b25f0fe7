/*
 * elbm_gb300 — C ABI of the GB300 (sm_103a) entropic lattice Boltzmann level step.
 *
 * The reference solver (University of Cincinnati Lattice Boltzmann Solver,
 * Fortran + AMReX) advances one AMR level per call chain
 *   streaming(level_step,fine,lvl)              looping/timestepping/streaming.f95:1
 *   calculate_flow_variables(level_step,fine,lvl) looping/timestepping/calculate_flow_variables.f95:1
 *   collision(level_step,fine,lvl)              looping/timestepping/collision.f95:1
 *   damp_it(level_step,fine,lvl)                looping/timestepping/damp_it.f95:1
 * issued from loop (looping/timestepping/loop.f95:94-147) over the boxes of the
 * level's MultiFabs (amr/modules/amr_info_holder.f95:70-76).  This library
 * replaces that chain with one fused device pass per level step.  The Fortran
 * driver keeps its subroutine signatures; their bodies call the functions
 * below through ISO_C_BINDING (fortran/elbm_gb300_iface.f90).
 *
 * Conventions
 *  - Plain pointers and sizes only.  Host arrays are AMReX FAB layouts: for a
 *    box lo..hi (inclusive, 0-based or not) with `ngrow` ghost layers the FAB
 *    spans (hi-lo+1+2*ngrow) nodes per axis, x fastest, then y, z, then the
 *    component (population) index — exactly mf%dataptr(mfi) of the reference.
 *  - Every call returns 0 on success or a negative ELBM_E_* code; it never
 *    aborts (the reference prints and STOPs, general/background_calcs/error_out.f95:12-14).
 *    elbm_last_error_string() describes the last failure.
 *  - One CUDA stream per context; a context is not thread-safe.  Steps are
 *    asynchronous; download and stats calls synchronise.
 */
#ifndef ELBM_GB300_H
#define ELBM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct elbm_ctx elbm_ctx;

/* return codes */
#define ELBM_OK 0
#define ELBM_E_ARG -1         /* bad argument (null pointer, size, ncomp) */
#define ELBM_E_CUDA -2        /* CUDA runtime error */
#define ELBM_E_UNSUPPORTED -3 /* unsupported link code / configuration */
#define ELBM_E_STATE -4       /* call out of order (e.g. step before upload) */
#define ELBM_E_NUMERIC -5     /* a set-up solve did not converge */

/* numerical health flags in elbm_stats.status */
#define ELBM_ST_NAN 0x1u             /* a density or velocity became NaN/Inf */
#define ELBM_ST_NEWTON_FALLBACK 0x2u /* some alpha solve fell back (count in .fallbacks) */
#define ELBM_ST_NEG_POP 0x4u         /* a post-collision population was negative */
#define ELBM_ST_DH_TOL 0x8u          /* check mode: some |dH| exceeded the tolerance */
#define ELBM_ST_COPY_TIMEOUT 0x10u   /* staged kernel: a bulk copy did not arrive in time; the step is invalid */

/* lattices */
#define ELBM_D3Q27 27
#define ELBM_D3Q39 39

/* population storage in HBM */
#define ELBM_STORE_FP64 0     /* f_i in FP64 */
#define ELBM_STORE_FP32_DEV 1 /* FP32 deviations d_i = f_i - w_i*rho0, rho0 = 1 */

/* entropic alpha */
#define ELBM_ALPHA_FIXED2 0  /* alpha = 2 (LBGK limit; calculate_flow_variables.f95:306-311 when turbulent is false) */
#define ELBM_ALPHA_NEWTON 1  /* Newton from alpha = 2 on H(f) = H(f + alpha*Delta) */
#define ELBM_ALPHA_LEARNED 2 /* MLP initial guess + at most two Newton polish steps, Newton fallback */

typedef struct {
  double nu;          /* kinematic viscosity (lattice units); beta = 1/(2 nu/T0 + 1), T0 = 1/3 */
  double tol_alpha;   /* Newton tolerance on alpha (FP64 path; 1e-12) */
  double tol_dH;      /* |H(f+alpha Delta) - H(f)| accepted by check mode and by the cap rule (1e-10) */
  int32_t max_newton; /* iteration cap */
  int32_t alpha_mode; /* ELBM_ALPHA_* */
  int32_t check_dH;   /* 1: evaluate |dH| per node in FP64 and report the maximum (validation runs) */
  int32_t record_alpha; /* 1: keep the per-node alpha of the last step for elbm_download_alpha */
  int32_t outlet_type[8]; /* per outlet number: 1,4 outlet eq; 2 inlet table; 3 freestream; 6 pure outflow */
  /* Boundary equilibria, computed by the host like
   * boundary_conditions/basic_calcs/freestream_basis_calcs.f90 and inlet_outlet_basis_calcs.f90 */
  double fs_feq[27];
  double inl_feq[8][27];
  double outl_feq[8][27];
  /* 1: every step repairs the negative post-collision populations it produced,
   * as damp_it.f95:64-177 does for unshifted lattices (see elbm_damp_level) */
  int32_t damp;
  int32_t pad_damp;
} elbm_d3q27_params;

/* D3Q39 compressible level: the reference's background scalars (computed by the
 * host like general/background_calcs/basic_fluids_calcs.f95, utilities/
 * viscosity_and_timing.f95 and general/background_calcs/timing_calcs.f95). */
typedef struct {
  int32_t shifted;           /* Galilean-shifted lattice (directions_and_weights.f95:477-499) */
  int32_t primary_flow_dir;  /* 1..6 */
  int32_t turbulent;         /* closed-form entropic alpha (calculate_alpha.f95:118-289), else alpha = 2 */
  int32_t lvl;               /* AMR level (beta_1 uses 2^(lvl+1)) */
  int32_t startup_timesteps; /* start-up ramps of beta, epsilon and alpha */
  int32_t max_lm_iters;      /* cap on the multiplier Newton (the reference has none) */
  int32_t periodic;          /* bit 0/1/2: x/y/z periodic; not 7 needs elbm_set_links39 */
  int32_t timestep;          /* timestep(amr_max_lvl) of the next step; advanced by elbm_level_step */
  int32_t damp;              /* 1: run the negative-population repair of damp_it.f95 after collision */
  int32_t pad;
  double gama, t_ref, rho_ref, p_ref, mu_ref, kappa_ref, gas_const_R, const_vol, const_press, molec_weight;
  double dt, elbm_epsilon, init_beta_1, init_beta_2, beta_1_scaling, beta_2_scaling;
  double su_lm[13];          /* start-up multipliers su_chi .. su_lambda_z (freestream_basis_calcs.f90:127-150):
                                the warm start next to interpolated walls in the first steps */
} elbm_d3q39_params;

typedef struct {
  int64_t node_updates;     /* fluid nodes advanced, summed over steps */
  int64_t newton_iters;     /* total Newton iterations (scalar or per-population) */
  int64_t exact_path_nodes; /* D3Q27 FP32 path: nodes with some |Delta_i/f_i| > 0.1 (solved out of line);
                               D3Q39 with damp = 1: negative f and g populations the repair met */
  int64_t fallbacks;        /* alpha solves that fell back */
  uint32_t status;          /* ELBM_ST_* flags */
  uint32_t pad;
  double max_abs_dH;        /* check mode only */
  int64_t dh_over_tol;      /* check mode: nodes whose |dH| exceeded tol_dH */
  int64_t guess_misses;     /* learned alpha: guesses that needed the Newton fallback from alpha = 2 */
  double kernel_ms;         /* device time of the step kernels (CUDA events) */
} elbm_stats;

/* Context on one CUDA device. */
int elbm_create(int device, elbm_ctx** out);
void elbm_destroy(elbm_ctx* ctx);
const char* elbm_last_error_string(const elbm_ctx* ctx);

/* Declare a level and its boxes.  Replaces the per-level MultiFab set-up of
 * from_scratch (amr/modules/amr_processes.f95:383-476).  lo_hi holds 6 ints per
 * box (lo x,y,z, hi x,y,z, inclusive).  ngrow is the ghost width of the
 * population FABs the host will pass (nghosts_mid in the reference,
 * general/background_calcs/directions_and_weights.f95:355-362).  Boxes must
 * not overlap.  A D3Q39 level of several boxes is held as one array over
 * their bounding box (links reach across box faces in place); its links,
 * populations, fields and initial state are complete once every box has been
 * given (elbm_set_links39, elbm_upload_level39 / elbm_upload_macro39,
 * elbm_init_level39).  An upload or initial state given to a box of a complete
 * level starts over: the level steps again once every box has been given anew. */
int elbm_level_register(elbm_ctx* ctx, int lvl, int lattice, int storage, int nbox, const int32_t* lo_hi,
                        int ngrow);

/* D3Q27 physical parameters and boundary equilibria of a level. */
int elbm_set_d3q27_params(elbm_ctx* ctx, int lvl, const elbm_d3q27_params* p);

/* D3Q39 scalars of a level (replaces the module globals the reference's
 * collision and flow-variable routines read). */
int elbm_set_d3q39_params(elbm_ctx* ctx, int lvl, const elbm_d3q39_params* p);

/* D3Q39 state of one box: fout, gout (39 comps), the 13 Lagrange multipliers
 * (chi, zeta_xyz, pi_xx,yy,zz,xy,xz,yz, lambda_xyz; 13 comps) and the previous
 * step's w velocity (1 comp), all as FABs with the level's ghost width. */
int elbm_upload_level39(elbm_ctx* ctx, int lvl, int box, const double* fout, const double* gout, const double* lm,
                        const double* w_vel);
/* Refinement tags of a D3Q39 box by the gradient of the gradient magnitude
 * of one macroscopic field (GGM/derivatives/calculate_grad_mag.f95 and
 * calculate_gradgrad_mag.f95, on the device from the fields the step keeps):
 * variable as populate_q.f95 numbers it (1 rho, 2 u, 3 v, 4 w, 5 pressure,
 * 6 T, 7 |u|, 8 0.5 rho |u|); scheme 0 central, 1 up-wind, 2 down-wind
 * differences (the namelist's central_diff / upwind_calculation /
 * downwind_calculation); limit: the level's ggm_tag_limit (the sensitivity
 * times 0.9^lvl, timing_calcs.f95:88-97).  tags (nx*ny*nz bytes, x fastest):
 * 1 where the node's GGM >= limit; ggm (may be NULL): the GGM values;
 * *ntagged (may be NULL): the tagged count. */
int elbm_ggm_tags(elbm_ctx* ctx, int lvl, int box, int variable, int scheme, double limit, uint8_t* tags, double* ggm,
                  int64_t* ntagged);
/* The same with predictive splitting (GGM/PGS/predictive_splitter.f95, the
 * namelist's pgs_on / pgs_reach) after the GGM tags: pgs_sensitivity is the
 * namelist's ggm_sensitivity (scan hits need ggm >= 2x, the isotropic case
 * 3x), pgs_reach the scan length in nodes (pgs_max_scan; < 0: no splitting).
 * The scans stay inside the box (the reference's reach also covers the FAB's
 * ghost nodes).  *ntagged counts every tag. */
int elbm_ggm_tags_pgs(elbm_ctx* ctx, int lvl, int box, int variable, int scheme, double limit, double pgs_sensitivity,
                      int pgs_reach, uint8_t* tags, double* ggm, int64_t* ntagged);

/* Plot3D output of a D3Q39 level from the device buffers, in the
 * reference's layout (output/plot3d_output.f95:77-215): Fortran unformatted
 * sequential records; grid file: block count, (nx, ny, nz) per block, then per
 * block x, y, z (4-byte reals: origin + (lo + i) dx) and blanks (1 node
 * type >= 0, -1 null node -666, 0 otherwise); data file: block count, the
 * dimensions with 6 variables and 0, then per block the header record and
 * rho, u, v, w, T, alpha (8-byte reals).  Every box of the level is a block. */
typedef struct {
  double mach, reynolds, time, gama, t_ref, stag_temperature, const_vol, const_press, non_dim_R;
} elbm_plot3d_header;
int elbm_write_plot3d(elbm_ctx* ctx, int lvl, const char* grid_path, const char* data_path, const double* origin,
                      double dx, const elbm_plot3d_header* hdr);
/* Microphones of a D3Q39 box (mic_write.f95:45-110): for each of nmic
 * microphones the weighted sums over its 8 nodes (box-local indices, x
 * fastest; weights from the microphone set-up) of pressure, T, rho, u, v, w,
 * gathered on the device; out: 6 values per microphone. */
int elbm_mic_sample(elbm_ctx* ctx, int lvl, int box, int nmic, const int32_t* nodes, const double* weights,
                    double* out);

/* Level checkpoints (restart; the reference's restart writer is commented
 * out, output/restart/restart_write.f95): the dynamic state of a level —
 * D3Q27: the post-collision populations; D3Q39, per box: f, g, the
 * multipliers, w, the macroscopic fields and, with link codes, the slots
 * that keep last step's values — and the D3Q39 timestep, written to one file
 * and read back bit for bit into a level registered, parameterised and
 * linked the same way.  No counterpart in the reference. */
int elbm_checkpoint_write(elbm_ctx* ctx, int lvl, const char* path);
int elbm_checkpoint_read(elbm_ctx* ctx, int lvl, const char* path);

/* Initial state of a D3Q39 box from its macroscopic fields rho, u, v, w, T
 * (5 comps, FAB layout), computed on the device node by node like
 * multilevel_initialization.f90:229-278: the multiplier Newton from lm_start
 * (13 values, e.g. the freestream start of freestream_basis_calcs.f90:24-90)
 * for rho, u and the equilibrium pressure tensor, then f = f_eq,
 * g = (2 C_v - 3) T f_eq; the multipliers, w and the fields are stored.
 * Replaces elbm_upload_level39 + elbm_upload_macro39 when the populations
 * start at equilibrium.  *capped (may be NULL): nodes whose Newton hit
 * max_lm_iters. */
int elbm_init_level39(elbm_ctx* ctx, int lvl, int box, const double* macro, const double* lm_start,
                      int64_t* capped);
/* The same solve for one state (rho, u, v, w, T in macro[5]), e.g. the
 * freestream or inlet equilibria elbm_set_links39 takes
 * (freestream_basis_calcs.f90): lm (13) is the start and returns the
 * multipliers; fieq, gieq receive 39 values each.  Uses the context's device;
 * no level needed.  ELBM_E_NUMERIC if the Newton does not converge. */
int elbm_d3q39_equilibrium(elbm_ctx* ctx, const elbm_d3q39_params* p, const double* macro, double* lm,
                           double* fieq, double* gieq);
/* The macroscopic fields rho, u, v, w, T (5 comps, FAB layout) the step
 * starts from: the reference's rho, u_vel, v_vel, w_vel, temp after
 * initialisation (multilevel_initialization.f90).  Needed by interpolated wall
 * links, which read the previous step's fields of the wall nodes and their
 * neighbours; call after elbm_upload_level39 (which clears them). */
int elbm_upload_macro39(elbm_ctx* ctx, int lvl, int box, const double* macro);
/* Any output pointer may be NULL.  macro: rho, u, v, w, T (5 comps). */
int elbm_download_level39(elbm_ctx* ctx, int lvl, int box, double* fout, double* gout, double* lm, double* w_vel,
                          double* alpha, double* macro);

/* Boundary data of a D3Q39 level with link codes (see elbm_set_links39):
 * inlet/outlet types per number (inlets 1, 2, 4: inlet table; 3: freestream;
 * outlets 1, 4: outlet table; 2: inlet table; 3: freestream; 6: pure outflow)
 * and the equilibria of f and g, computed by the host like
 * freestream_basis_calcs.f90 and inlet_outlet_basis_calcs.f90. */
typedef struct {
  int32_t inlet_type[8], outlet_type[8];
  double fs_fieq[39], fs_gieq[39];
  double inl_fieq[8][39], inl_gieq[8][39];
  double outl_fieq[8][39], outl_gieq[8][39];
  double fs_u, fs_v, fs_w, fs_temp; /* freestream velocity and temperature (fs_u .. temperature of the
                                       reference), read by the interpolated wall links */
} elbm_d3q39_bc;

/* Link codes of a D3Q39 box (state FAB, 39 comps, ngrow_state ghosts), for
 * levels that are not periodic on every axis.  The library works out, for
 * every node and population, what the reference's push loop
 * (streaming.f95:266-481: direction outermost, boundary rules applied to fout
 * in place before fi is written, the interior push as well on the shifted
 * lattice) leaves in the post-streaming slot: a population of a node within 4
 * links, a boundary equilibrium, or the slot's value of the previous step.
 * Supported codes: >= 0, -5, -8, -10, -100-k, -200-k, -300-k, -400-k, -666,
 * -1000, the interpolated wall links -1001 - floor(q 1e9) (the targets of
 * target_finder.f95, then the Grad-type closure of shifted_ibb.f95 on the
 * shifted lattice with primary_flow_dir 1, or the per-direction closure of
 * interpolative_bounceback_bc.f95:834-2838 on the unshifted lattice, whose
 * value of link i is streamed into slot opp(i); they read the previous step's
 * macroscopic fields, so elbm_upload_macro39 must follow elbm_upload_level39), and the
 * inviscid links -11 / -12 (specular reflection of inviscid_edge.f95: the
 * population goes to the mirror direction at a displaced node; an inviscid
 * link needs a -11 among the node's unit or speed-2 axis links, which the
 * reference's table selects on).  Nodes with state < 0 neither
 * push nor collide; state >= 0 must be fluid (outside 200..298 and
 * 1000..50999); nodes outside the box on a non-periodic axis count as null
 * nodes (-666), as lbgrid/fluid_or_solid.f95:69-119 marks them for an
 * external flow.  With damp = 1 the fout and gout parts of damp_it.f95
 * follow every step with the rules for boundary links (unshifted: interior
 * links select the neighbours; shifted: the band near the box's high faces
 * and the node types >= -500; outside the box each set's freestream
 * equilibrium); its fi and gi parts, which only matter for slots no rule
 * writes, are not applied. */
int elbm_set_links39(elbm_ctx* ctx, int lvl, int box, const int32_t* state, int ngrow_state,
                     const elbm_d3q39_bc* bc);

/* The tables elbm_set_links39 builds, on the host only (no device, no
 * context): per node a type (0 neither pushes nor collides, 1 plain pulls,
 * 2 boundary record, 3 boundary record with interpolated wall links) and, for
 * each of the *nrec records (at most capacity), the node and 39 link words
 * (bits 0-1 kind: 0 previous post-streaming value, 1 pull, 2 equilibrium,
 * 3 interpolated wall value; bits 2-7 population; 8-12 table; 13-22 offset
 * (dx+4) + 9(dy+4) + 81(dz+4)).  For inspection and tests. */
int elbm_links39_tables(int nx, int ny, int nz, const int32_t* state, int ngrow_state, int periodic, int shifted,
                        int primary_flow_dir, const int32_t* inlet_type, const int32_t* outlet_type, uint8_t* ntype,
                        int32_t* rec_node, uint32_t* words, int64_t capacity, int64_t* nrec);

/* Node types and link codes of one box: the reference's integer `state` FAB
 * (Q components, ghost width ngrow_state; encoding of looping/timestepping/loop.f95:71-89,
 * case ranges of streaming.f95:365-481).  Decoded once into a node-type byte
 * per node and a compact table of boundary links. */
int elbm_set_links(elbm_ctx* ctx, int lvl, int box, const int32_t* state, int ngrow_state);

/* Set-up helper (host code, no GPU): mark the solid nodes of a closed
 * triangulated surface (ray casting, like lbgrid/fluid_or_solid) and the wall
 * links of the fluid nodes with their packed crossing fraction
 * state = -1001 - floor(|x - x_w| / (|c_i| dx) * 1e9), the encoding of
 * lbgrid/inter_bb_setup.f95:44-246 and linking/modules/linkwise.f95:45-57.
 * state: 27 components of nx*ny*nz int32 (no ghosts), updated in place; node
 * (i,j,k) sits at origin + (i,j,k)*dx; tri: 9 doubles per triangle. */
int elbm_mark_triangles(int nx, int ny, int nz, const double* origin, double dx, int ntri, const double* tri,
                        int32_t* state);
/* The same marking on the context's device (a block per +x ray for the
 * solid test, a thread per node for the wall links, the uniform triangle grid
 * built on the host): the same codes bit for bit, the set-up cost of large
 * levels moved off the host (ELBM_E_UNSUPPORTED when more than 4096 triangles
 * meet one +x ray; elbm_mark_triangles handles those). */
int elbm_mark_triangles_gpu(elbm_ctx* ctx, int nx, int ny, int nz, const double* origin, double dx, int ntri,
                            const double* tri, int32_t* state);
/* The D3Q39 codes of a box from a closed triangulated surface (the same set-up
 * for the D3Q39 lattices: lbgrid/shifted_state_directions.f95:54-68 on the
 * shifted lattice, state_directions.f95:696 on the unshifted one, with the
 * crossing of inter_bb_setup.f95 / linkwise.f95:45-57).  state is
 * (39, nz, ny, nx), updated in place: solid nodes (odd count of +x ray
 * crossings) get node type -1001 and -666 on their links; link i of a fluid
 * node gets -1001 - floor(t 1e9) when the node x - c_i (shifted lattice, c the
 * shifted velocities of primary_flow_dir) or x + c_i (unshifted) is solid, t
 * the nearest crossing of the segment towards it (1 when none is found);
 * periodic (bits x, y, z) wraps that neighbour.  elbm_mark_triangles39 runs on
 * the host, elbm_mark_triangles39_gpu on the context's device with the same
 * codes bit for bit. */
int elbm_mark_triangles39(int nx, int ny, int nz, const double* origin, double dx, int ntri, const double* tri,
                          int shifted, int primary_flow_dir, int periodic, int32_t* state);
int elbm_mark_triangles39_gpu(elbm_ctx* ctx, int nx, int ny, int nz, const double* origin, double dx, int ntri,
                              const double* tri, int shifted, int primary_flow_dir, int periodic, int32_t* state);

/* Copy one box's post-collision populations (fout FAB, FP64, Q comps) to / from the device. */
int elbm_upload_level(elbm_ctx* ctx, int lvl, int box, const double* fout);
int elbm_download_level(elbm_ctx* ctx, int lvl, int box, double* fout);

/* Allocation-free variant of elbm_upload_level for D3Q27 levels with FP32
 * deviation storage.  No counterpart in the reference: it exists for callers
 * that cannot let the library allocate device memory once the level is set
 * up, such as an AMReX driver whose arena has already reserved the GPU's
 * memory, or a time loop that must not stall on cudaMalloc's device-wide
 * synchronisation.  The FP64 FAB is staged through a fixed 32 MiB buffer built
 * into the library (held by every GPU that loads it, until exit) instead of a
 * cudaMalloc'ed one; boxes needing more than 32 MiB of FP64 populations
 * (27 x nodes x 8 bytes, i.e. more than 155,344 nodes) are rejected with
 * ELBM_E_ARG.  The buffer is reserved, and its address looked up, when a
 * context is created on the device (elbm_create), so this call loads nothing
 * and allocates nothing.  All calls share the buffer and it keeps the last
 * call's contents (each call overwrites what it reads): calls that overlap on
 * the GPU race.  The call returns after the copy has finished. */
int elbm_upload_level_noalloc(elbm_ctx* ctx, int lvl, int box, const double* fout);

/* Per-node alpha of the last step (valid-box layout without ghosts, FP64). */
int elbm_download_alpha(elbm_ctx* ctx, int lvl, int box, double* alpha);

/* Advance the level by nsteps fused steps (stream + boundaries + moments +
 * alpha + collision).  Replaces streaming/calculate_flow_variables/collision
 * for one level (looping/timestepping/loop.f95:104-139).  stats may be NULL;
 * when given, the call synchronises and fills it. */
int elbm_level_step(elbm_ctx* ctx, int lvl, int nsteps, elbm_stats* stats);

/* Coarse-fine transfer between D3Q27 levels lvl - 1 (coarse) and lvl (fine),
 * refinement ratio 2, nodal indexing (fine node X lies on coarse node X/2).
 * Fine nodes whose state is a ghost code (1e7 .. 1.1e9) belong to the fine
 * level's boxes, are stepped like fluid nodes, and are refilled from the
 * coarse level.  Replaces interlevel_interpolation.f95:114-440 and
 * fine_to_coarse.f95:13-64 for two D3Q27 levels of one storage or two D3Q39
 * levels (both with link codes, elbm_set_links39).
 *   elbm_interlevel_setup: build the maps, after both levels' links.
 *   elbm_fill_fine_ghosts: explosion, every fine ghost node <- nodal bilinear
 *     interpolation of the coarse populations.  D3Q27: a negative or NaN
 *     population sends the node to the entropic equilibrium of the
 *     interpolated moments.  D3Q39: f, g, the 13 multipliers, rho and T are
 *     interpolated; each population with f < 0, g < 0 or NaN takes the coarse
 *     equilibrium f_eq(rho_c, lm_c), g = (2 C_v - 3) T_c f; then the node's
 *     moments, its multiplier Newton from the interpolated multipliers and its
 *     alpha are stored (the coarse level needs its fields: a step,
 *     elbm_upload_macro39 or elbm_init_level39).  repaired (may be NULL):
 *     ghost nodes with a replaced population; with repaired non-NULL a D3Q39
 *     multiplier solve that hit the iteration cap returns ELBM_E_NUMERIC.
 *   elbm_average_down: coalescence, coarse nodes under valid fine nodes <-
 *     the fine populations (nodal injection; D3Q39 also g, multipliers, w,
 *     alpha and the fields).
 * Both act on the current (post-collision) populations; the driver calls
 * them where the reference calls interlevel_interpolation and fine_to_coarse
 * (loop.f95:116-128), on the sub-steps the reference does. */
int elbm_interlevel_setup(elbm_ctx* ctx, int lvl);
int elbm_fill_fine_ghosts(elbm_ctx* ctx, int lvl, int64_t* repaired);
int elbm_average_down(elbm_ctx* ctx, int lvl);

/* Advance D3Q27 levels 0 .. nlev-1 by ncycles coarse steps with 2:1
 * sub-cycling (level l steps 2^l times per coarse step), the fine levels
 * refilled from their coarse level before the first of their two steps
 * completes and averaged down after the second, as in loop.f95:94-147.  The
 * launches of two coarse cycles are captured once in a CUDA graph and
 * replayed (the capture is redone when the levels' buffers, parameters or
 * kernel variant change).  stats covers all levels (may be NULL).  No
 * counterpart in the reference (its loop issues each phase from the host). */
int elbm_amr_run(elbm_ctx* ctx, int nlev, int ncycles, elbm_stats* stats);

/* Repair the negative populations of a D3Q27 level's current post-collision
 * state, as damp_it.f95:64-177 (unshifted lattice): a negative f_i at x takes
 * the mean of f_i(x + c_i) and f_i(x - c_i) when both links from x are fluid
 * links and both values positive; with one positive fluid-link neighbour, the
 * mean of it and |f_i|; otherwise |f_i|.  Neighbours are read before any
 * repair (the reference repairs in place, so the two differ only when two
 * negative populations of one direction are adjacent along c_i).  repaired
 * (may be NULL) receives the number of populations changed; a level holds at
 * most 2^22 pending repairs per call (more: ELBM_E_STATE, nothing changed). */
int elbm_damp_level(elbm_ctx* ctx, int lvl, int64_t* repaired);

/* Time every variant of the level's step kernel on its current state (reps
 * launches each, the state does not advance) and keep the fastest for
 * elbm_level_step.  chosen and ms_per_variant (room for ELBM_KERNEL_VARIANTS)
 * may be NULL.  The reference has no counterpart (it has one code path per
 * lattice). */
#define ELBM_KERNEL_VARIANTS 10
int elbm_autotune(elbm_ctx* ctx, int lvl, int reps, int* chosen, double* ms_per_variant);

/* Use kernel variant v (0: direct loads; 1, 4, 5, 6, 7: direct, registers
 * capped for 4, 5, 6, 8, 7 blocks of 128 threads per SM; 2: rows staged in
 * shared memory by bulk copies, persistent; 3: direct loads, persistent warps
 * taking 32-node chunks from a counter; 8: warp-specialised, a producer warp
 * keeps tensor copies (TMA) of 256-node tiles in flight into a shared-memory
 * ring while eight consumer warps collide; 9: direct loads at 27 offsets
 * computed once per launch, for one-box levels whose 27 population planes
 * stay below 2^31 elements) for the level's FP32 D3Q27 steps,
 * instead of the autotuner's choice.  Variant 2 applies to boxes with nx and
 * the plane size multiples of 4 and ny, nz >= 3, other boxes fall back to
 * variant 0; variant 8 serves FP32 levels whose boxes all have nx a multiple
 * of 4, and asking for it (or for 9 on a level it does not serve) on another
 * level returns ELBM_E_UNSUPPORTED with the reason in elbm_last_error_string.
 * No counterpart in the reference. */
int elbm_set_kernel_variant(elbm_ctx* ctx, int lvl, int variant);

/* Learned initial guess of alpha (no counterpart in the reference; its
 * Future Work.txt:34 proposes machine learning to shorten the solves): a
 * 27-64-64-1 GELU network maps y/lambda (y_i = Delta_i/f_i, lambda = max|y_i|)
 * to (alpha - 2)/lambda.  Weights: 6017 floats, W1[27][64], b1[64], W2[64][64],
 * b2[64], w3[64], b3.  Records: 29 floats, y/lambda (27), lambda, target. */
#define ELBM_MLP_PARAMS 6017
#define ELBM_MLP_RECORD 29

/* Run nsteps Newton-alpha steps of an FP32 D3Q27 level and collect a record
 * from every stride-th node whose solve converged (at most capacity). */
int elbm_alpha_harvest(elbm_ctx* ctx, int lvl, int nsteps, int stride, float* records, int64_t capacity,
                       int64_t* count);
/* Mean-squared-error loss and its gradient for one batch (the training kernels). */
int elbm_alpha_mlp_grad(elbm_ctx* ctx, const float* weights, const float* records, int64_t n, float* grad,
                        double* loss);
/* Network outputs for n feature rows (27 floats each: y/lambda) by the
 * tensor-core inference the learned-alpha step uses (BF16 operands, FP32
 * accumulation, 128 rows per tile).  status (may be NULL) receives
 * ELBM_ST_COPY_TIMEOUT if a tile's matrix multiply did not complete. */
int elbm_alpha_mlp_infer(elbm_ctx* ctx, const float* weights, const float* x, int64_t n, float* out,
                         uint32_t* status);
/* Adam training on the GPU; weights in/out; loss_per_epoch may be NULL. */
int elbm_alpha_mlp_train(elbm_ctx* ctx, const float* records, int64_t n, int epochs, int batch, float lr,
                         uint64_t seed, float* weights, double* loss_per_epoch);
/* Weights used by ELBM_ALPHA_LEARNED on this level. */
int elbm_set_alpha_mlp(elbm_ctx* ctx, int lvl, const float* weights);

/* Wait for all work of the context. */
int elbm_sync(elbm_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* ELBM_GB300_H */
