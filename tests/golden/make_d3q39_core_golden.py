"""Golden values of the D3Q39 core, run straight from the reference's own
Fortran statements (tests/golden/f95_subset.py interprets them in float64):

  lattice tables        general/background_calcs/directions_and_weights.f95 (D3Q39 branch)
  equilibrium           amr/modules/amr_processes.f95 fieq_comp_39, fieq_comp_39_shifted
  multiplier solve      looping/timestepping/lagrangian_multipliers/calculate_lagrangian_mults.f95
                        (unshifted hand-expanded Jacobian :341-695, shifted generic :696-1097)
  LU update             looping/timestepping/lagrangian_multipliers/lu_decomp.f95 (both index quirks)
  closed-form alpha     looping/timestepping/calculate_alpha.f95
  heat-flux corrections looping/timestepping/component_subroutines/find_q_bar.f95, find_little_q_bar.f95
  flow variables        looping/timestepping/calculate_flow_variables.f95:192-228 (moments of f and g,
                        temperature, pressure and the six pressure-tensor targets; P_zz reads the stored w)
  collision of a node   looping/timestepping/collision.f95 (the body of the per-node loop)
  wall targets          boundary_conditions/interpolative_bc/target_finder.f95 (both lattices)
  shifted wall closure  boundary_conditions/interpolative_bc/shifted_ibb.f95 with the wall and local
                        derivatives of derivatives/modules/derivatives.f95
  push loop             looping/timestepping/streaming.f95:263-1161 with the boundary routines it calls
                        (bc_switchboard, bounceback, inlet_bc, outlet_bc and its variants,
                        freestream_edge_bc, inviscid_edge; on the wall cases also target_finder, the target
                        multiplier solve and shifted_ibb) on boxes of push39_inputs: digests of the
                        post-streaming fi, gi of the fluid nodes (the wall-link slots, whose closure sums
                        the oracle orders its own way, as values), written to d3q39_push_golden.json
  explosion of a node   looping/timestepping/interlevel/interlevel_interpolation.f95 (the per-node block
                        after the interpolation: coarse equilibrium for negative or NaN pairs, moments,
                        multiplier solve, alpha)
  GGM derivative        derivatives/modules/derivatives.f95:589-700 (derivative_windage_secondord and
                        _firstord: central, upwind and downwind schemes)
  gradient tags         GGM/derivatives/calculate_grad_mag.f95, calculate_gradgrad_mag.f95 (three schemes)
  predictive splitting  GGM/PGS/predictive_splitter.f95 (the loop over a box of pgs_inputs; ghost
                        layers of node type -666, which no scan counts)
  fout repair           looping/timestepping/damp_it.f95 (the reach and the in-place sweep of one box,
                        fout and gout parts, written to d3q39_damp_golden.json)
  transport             utilities/modules/quick_calcs.f95, amr_processes.f95 beta_1/2_calculator,
                        epsilon_calculator

Each case records its inputs and the reference's outputs; tests/test_oracle_d3q39_golden.py
runs the oracle's restatement on the same inputs.  The constants of a case (reference scales,
relaxation ramps) come from the package's host set-up of the wedge case (d3q39_setup), which
restates basic_fluids_calcs / viscosity_and_timing; they are inputs here and are stored with the
case.

Two statements of streaming.f95 are rewritten for the interpreter without changing what runs
(see Reference.push), and three facts of the reference's set-up are stated rather than run:
directions_and_weights sets nghosts_mid before it sets `shifted`, so the module's initial .false.
gives nghosts_mid = 8; the periodic span and AMReX's ghost images are left out of the push boxes
(their sweep order is a documented difference); the fi and gi parts of damp_it see positive values.

Run: python make_d3q39_core_golden.py <reference root>
     (writes d3q39_core_golden.json, d3q39_damp_golden.json and d3q39_push_golden.json)
"""
from __future__ import annotations

import importlib.util
import json
import math
import pathlib
import re
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import damp39_inputs  # noqa: E402
import pgs_inputs  # noqa: E402
import push39_inputs  # noqa: E402
import f95_subset as F  # noqa: E402

PKG = HERE.parents[1] / "university-of-cincinnati-lattice-boltzmann-solver_gb300"

CONST_FIELDS = ("shifted", "primary_flow_dir", "turbulent", "lvl", "startup_timesteps", "max_lm_iters", "gama",
                "t_ref", "rho_ref", "p_ref", "mu_ref", "kappa_ref", "gas_const_R", "const_vol", "const_press",
                "molec_weight", "dt", "elbm_epsilon", "init_beta_1", "init_beta_2", "beta_1_scaling",
                "beta_2_scaling")
LM_NAMES = ("chi", "zeta_x", "zeta_y", "zeta_z", "pi_xx", "pi_yy", "pi_zz", "pi_xy", "pi_xz", "pi_yz", "lambda_x",
            "lambda_y", "lambda_z")


def _setup_module():
    spec = importlib.util.spec_from_file_location("d3q39_setup", PKG / "d3q39_setup.py")
    m = importlib.util.module_from_spec(spec)
    sys.modules["d3q39_setup"] = m
    spec.loader.exec_module(m)
    return m


def _module_values(path: pathlib.Path, out: dict):
    """Initialised module variables and PARAMETERs of a module file, in order."""
    interp = F.Interp({}, {})
    sc = F.ChainMap(out, F.INTRINSICS)
    for no, s in F.logical_lines(path.read_text()):
        if "::" in s and "=" in s.split("::", 1)[1] and F._DECL.match(s):
            interp.declare(s, out, sc, set())


def _int_arrays(*paths):
    """Names of the INTEGER allocatable arrays declared in module files."""
    names = set()
    for p in paths:
        for no, s in F.logical_lines(p.read_text()):
            m = re.match(r"^integer\b[^:]*allocatable[^:]*::(.*)$", s)
            if m:
                for item in F.split_top(m.group(1)):
                    names.add(re.match(r"(\w+)", item).group(1))
    return names


class Reference:
    """The reference's routines with the module state of one lattice and case."""

    def __init__(self, root: pathlib.Path, c, shifted: bool):
        R = root
        files = [R / "amr/modules/amr_processes.f95",
                 R / "looping/timestepping/lagrangian_multipliers/calculate_lagrangian_mults.f95",
                 R / "looping/timestepping/lagrangian_multipliers/lu_decomp.f95",
                 R / "looping/timestepping/calculate_alpha.f95",
                 R / "looping/timestepping/component_subroutines/find_q_bar.f95",
                 R / "looping/timestepping/component_subroutines/find_little_q_bar.f95",
                 R / "utilities/modules/quick_calcs.f95",
                 R / "general/background_calcs/directions_and_weights.f95",
                 R / "boundary_conditions/interpolative_bc/target_finder.f95"] + \
                [R / "boundary_conditions" / f for f in ("bc_switchboard.f95", "bounceback.f95", "inlet_bc.f95",
                                                          "outlet_bc.f95", "rho_v_bc.f95", "press_temp_bc.f95",
                                                          "v_temp_bc.f95", "freestream_bc.f95", "null_bc.f95",
                                                          "freestream_edge_bc.f95", "pure_outflow_bc.f95",
                                                          "inviscid_edge.f95")]
        wanted = {"fieq_comp_39", "fieq_comp_39_shifted", "beta_1_calculator", "beta_2_calculator",
                  "epsilon_calculator", "calculate_lagrangian_mults", "lu_decomp", "calculate_alpha", "find_q_bar",
                  "find_little_q_bar", "quick_sutherlands", "quick_therm_cond", "directions_and_weights",
                  "target_finder", "bc_switchboard", "bounceback", "inlet_bc", "outlet_bc", "rho_v_bc",
                  "press_temp_bc", "v_temp_bc", "freestream_bc", "null_bc", "freestream_edge_bc", "pure_outflow_bc",
                  "inviscid_edge"}
        self.procs = {}
        for p in files:
            self.procs.update(F.parse_units(F.logical_lines(p.read_text()), only=wanted))
        # the wall-derivative functions of the derivatives module (shifted_ibb's stencil)
        self.procs.update(F.parse_units(F.logical_lines((R / "derivatives/modules/derivatives.f95").read_text())))
        ibb = ("shifted_ibb", "shifted_ibb.f95") if shifted else \
            ("interpolative_bounceback_bc", "interpolative_bounceback_bc.f95")
        self.procs.update(F.parse_units(F.logical_lines(
            (R / "boundary_conditions/interpolative_bc" / ibb[1]).read_text()), only={ibb[0]}))
        missing = wanted - set(self.procs)
        if missing:
            raise RuntimeError(f"reference routines not found: {sorted(missing)}")
        g = {"dp": F.FInt(8), "sp": F.FInt(4)}
        _module_values(R / "general/modules/precise.f95", g)
        _module_values(R / "general/modules/constants.f95", g)
        _module_values(R / "linking/modules/linkwise.f95", g)  # erp, the unshifted opposites
        # case values of the modules (constants, timing, amr_info_holder, grid_data, namelists)
        g.update(dimensions=F.FInt(3), primary_flow_dir=F.FInt(c.primary_flow_dir), gama=c.gama, t_ref=c.t_ref,
                 rho_ref=c.rho_ref, p_ref=c.p_ref, mu_ref=c.mu_ref, kappa_ref=c.kappa_ref, gas_const_r=c.gas_const_R,
                 const_vol=c.const_vol, const_press=c.const_press, molec_weight=c.molec_weight,
                 init_beta_1=c.init_beta_1, init_beta_2=c.init_beta_2, beta_1_scaling=c.beta_1_scaling,
                 beta_2_scaling=c.beta_2_scaling, startup_timesteps=F.FInt(c.startup_timesteps),
                 self=F.FInt(0), amr_max_lvl=F.FInt(0), mach=(1.5 if shifted else 0.5), use_shifted=bool(shifted),
                 shifted=bool(shifted), turbulent=True,
                 temperature=c.temperature,
                 dt=F.FArray(np.array([c.dt]), [0]), elbm_epsilon=F.FArray(np.array([c.elbm_epsilon]), [0]),
                 timestep=F.FArray(np.array([0], np.int64), [0]))
        g["__int_arrays"] = _int_arrays(R / "linking/modules/linkwise.f95") | {"opp"}
        self.interp = F.Interp(self.procs, g)
        self.g = g
        self.interp.call("directions_and_weights", [])
        assert int(g["dir"]) == 39 and bool(g["shifted"]) == bool(shifted)
        self.lu_log = []
        real_lu = self.real_lu = self.procs["lu_decomp"]

        def val(a):
            return a.get() if isinstance(a, F.Ref) else a

        def lu_hook(*acts):
            jac = np.array(val(acts[0]).a, copy=True)
            moments = [float(val(a)) for a in acts[2:15]]
            lm_in = [float(val(r)) for r in acts[15:28]]
            self.interp.call_proc(real_lu, list(acts))
            lm_out = [float(val(r)) for r in acts[15:28]]
            self.lu_log.append({"jacobian": jac.ravel().tolist(), "moments": moments, "lm_in": lm_in,
                                "lm_out": lm_out, "max_diff": float(val(acts[28]))})
            if len(self.lu_log) > 200:
                raise RuntimeError("multiplier solve did not converge in 200 iterations")

        self.procs["lu_decomp"] = self._lu_hook = lu_hook

    def set_step(self, step: int):
        self.g["timestep"].set((0,), step)

    def tables(self):
        return {k: [int(v) for v in self.g[k].a] for k in ("cx", "cy", "cz", "opp")}

    def fieq(self, rho, lm):
        name = "fieq_comp_39_shifted" if self.g["shifted"] else "fieq_comp_39"
        return [float(self.interp.call(name, [rho] + list(lm) + [F.FInt(i)])) for i in range(1, 40)]

    def lagrange(self, rho, u, v, w, T, P, lm0):
        self.lu_log = []
        lm = {n: float(x) for n, x in zip(LM_NAMES, lm0)}
        fe = F.FArray(np.full(39, np.nan))
        acts = [rho, u, v, w, T] + list(P) + [F.Ref(lm, n) for n in LM_NAMES] + [fe, F.FInt(1), F.FInt(1),
                                                                                   F.FInt(1)]
        self.interp.call("calculate_lagrangian_mults", acts)
        return [lm[n] for n in LM_NAMES], fe.a.tolist(), list(self.lu_log)

    def alpha(self, fi, fd, T):
        out = {"a": float("nan")}
        fi4 = F.FArray(np.asarray(fi, np.float64).reshape(1, 1, 1, 39), [1, 1, 1, 1])
        self.interp.call("calculate_alpha", [fi4, F.FArray(np.asarray(fd, np.float64)), F.Ref(out, "a"), T,
                                             F.FInt(0), F.FInt(0), F.FInt(1), F.FInt(1), F.FInt(1)])
        return out["a"]

    def q_bar(self, fd, fe, u, v, w, T):
        qb = F.FArray(np.full(39, np.nan))
        self.interp.call("find_q_bar", [F.FArray(np.asarray(fd, np.float64)), F.FArray(np.asarray(fe, np.float64)),
                                        qb, u, v, w, T, F.FInt(0)])
        return qb.a.tolist()

    def little_q_bar(self, gd, u, v, w, T):
        ch = F.FArray(np.full(39, np.nan))
        self.interp.call("find_little_q_bar", [F.FArray(np.asarray(gd, np.float64)), u, v, w, T, ch, F.FInt(0)])
        return ch.a.tolist()

    def flow_vars(self, root, f, g, w_old):
        """calculate_flow_variables.f95's statements for one node (a = b = c = 1) from the
        sums of f and g (:192) to the last pressure-tensor target (:228), just before the
        multiplier solve; w_old is the node's stored w, which the P_zz target reads."""
        lines = F.logical_lines((root / "looping/timestepping/calculate_flow_variables.f95").read_text())
        i0 = next(k for k, (no, s) in enumerate(lines) if re.match(r"^rho_sum\s*=", s))
        body, _ = F.parse_block(lines, i0, r"^if\s*\(timestep\(lvl\)")
        local = {}
        scope = self.interp.scope_for(local)
        for no, s in lines[:i0]:
            if re.match(r"^(real|integer)\b", s) and "intent" not in s:
                self.interp.declare(s, local, scope, set())

        def node_arr(vals):
            a = np.asarray(vals, np.float64).reshape(1, 1, 1, -1)
            return F.FArray(a.copy(), [1, 1, 1, 1])

        nan = [float("nan")]
        local.update(a=F.FInt(1), b=F.FInt(1), c=F.FInt(1), lvl=F.FInt(0), fi=node_arr(f), gi=node_arr(g),
                     rho=node_arr(nan), u_vel=node_arr(nan), v_vel=node_arr(nan), w_vel=node_arr([w_old]),
                     temp=node_arr(nan), press=node_arr(nan))
        self.interp.run(body, local, scope)
        one = lambda name: float(local[name].a.ravel()[0])  # noqa: E731
        return [one("rho"), one("u_vel"), one("v_vel"), float(local["dummy_w"]), one("temp"),
                float(local["new_pxx"]), float(local["new_pyy"]), float(local["new_pzz"]), float(local["new_pxy"]),
                float(local["new_pxz"]), float(local["new_pyz"]), one("press")]

    def push(self, root, cs, G=8):
        """streaming.f95's push loop (:263-1161) over one box at level 0, for a case of
        push39_inputs (boundary links, no interpolated wall links).  The box's FABs get G
        ghost layers: on a periodic axis the periodic images (as fill_boundary leaves
        them), on the others nodes whose every code is -666 (outside an external-flow
        domain).  Two statements are rewritten for the interpreter, neither changing what
        runs: `go to 1000` (the shifted lattice's rest-direction push onto a fluid node)
        becomes the two assignments labelled 1000 followed by `cycle` (after the SELECT
        nothing but a diagnostic print remains in the loop body), and the box bounds
        wax%lo, wax%hi become the arrays wax_lo, wax_hi.  fi, gi start from the previous
        step's post-streaming values (what slots no rule writes keep).  Returns the
        post-streaming fi, gi of the box, (39, nz, ny, nx)."""
        text = (root / "looping/timestepping/streaming.f95").read_text()
        label_line = next(no for no, s in enumerate(text.splitlines(), 1) if re.match(r"^\s*1000\s+fi\(", s))
        raw = F.logical_lines(text)  # (statement labels are dropped there)
        k_goto = next(k for k, (no, s) in enumerate(raw) if re.match(r"^go\s*to\s+1000$", s))
        k_lab = next(k for k, (no, s) in enumerate(raw) if no == label_line)
        lab_f, lab_g = raw[k_lab][1], raw[k_lab + 1][1]
        assert lab_f.startswith("fi(a+cx(i)") and lab_g.startswith("gi(a+cx(i)"), (lab_f, lab_g)
        lines = []
        for k, (no, s) in enumerate(raw):
            s = s.replace("wax%lo(", "wax_lo(").replace("wax%hi(", "wax_hi(")
            lines += [(no, lab_f), (no, lab_g), (no, "cycle")] if k == k_goto else [(no, s)]
        k_reach = next(k for k, (no, s) in enumerate(lines) if s == "if (.not. shifted) then")
        k_kg = next(k for k, (no, s) in enumerate(lines) if s.startswith("k_gieq = "))
        k_pt = next(k for k, (no, s) in enumerate(lines) if s == "node_pt = 0")
        k_loop = next(k for k in range(k_pt, len(lines)) if re.match(r"^do\s+i\s*=\s*1\s*,\s*dir$", lines[k][1]))
        reach_if, _ = F.parse_stmt(lines, k_reach)
        kg_stmt, _ = F.parse_stmt(lines, k_kg)
        loop, _ = F.parse_stmt(lines, k_loop)
        st = cs["state"]
        q, nz, ny, nx = st.shape
        per_y = bool(cs["periodic"] & 2)

        def fab(arr, fill, dtype):
            out = np.full((nx + 2 * G, ny + 2 * G, nz + 2 * G, 39), fill, dtype)
            t = np.transpose(arr, (3, 2, 1, 0))
            out[G:G + nx, G:G + ny, G:G + nz, :] = t
            if per_y:
                for yf in list(range(G)) + list(range(G + ny, ny + 2 * G)):
                    out[G:G + nx, yf, G:G + nz, :] = t[:, (yf - G) % ny, :, :]
            return out

        lb = [-G, -G, -G, 1]
        g = self.g
        g["inlet_type"] = F.FArray(np.array([cs["inlet_type"], cs["inlet_type"]], np.int64), [1, 1])
        g["outlet_type"] = F.FArray(np.array([cs["outlet_type"], cs["outlet_type"]], np.int64), [1, 1])
        g["inl_fieq"] = F.FArray(np.array([cs["fi"]] * 8).T.copy(), [1, 1])
        g["inl_gieq"] = F.FArray(np.array([cs["gi"]] * 8).T.copy(), [1, 1])
        g["outl_fieq"] = F.FArray(np.array([cs["fo"]] * 8).T.copy(), [1, 1])
        g["outl_gieq"] = F.FArray(np.array([cs["go"]] * 8).T.copy(), [1, 1])
        g["fs_fieq"] = F.FArray(np.asarray(cs["ff"], np.float64).copy(), [1])
        g["fs_gieq"] = F.FArray(np.asarray(cs["gf"], np.float64).copy(), [1])
        local = {}
        scope = self.interp.scope_for(local)
        self.interp.declare("integer :: a,b,c,i,j,reach,loc_cx,loc_cy,loc_cz,fine,state_pass(7)", local, scope,
                            set())
        self.interp.declare("real(kind=dp) :: loc_fieq,loc_gieq,loc_fieq_opp,loc_gieq_opp,k_gieq,pass_fieq(dir),"
                            "pxx_temp,pyy_temp,pzz_temp,pxy_temp,pxz_temp,pyz_temp", local, scope, set())
        for nm in ("u_local", "v_local", "w_local", "temp_local"):
            local[nm] = F.FArray(np.zeros(7))
        for nm in ("u_pass", "v_pass", "w_pass", "temp_pass"):
            local[nm] = F.FArray(np.zeros(39))
        if "fields" in cs:
            # the fields, multipliers and the per-node target scratch FABs the wall branch reads and writes
            def fab1(arr3):
                out = np.zeros((nx + 2 * G, ny + 2 * G, nz + 2 * G, 1))
                out[G:G + nx, G:G + ny, G:G + nz, 0] = np.transpose(arr3, (2, 1, 0))
                return F.FArray(out, lb)
            for nm, arr in zip(("rho", "u_vel", "v_vel", "w_vel", "temp"), cs["fields"]):
                local[nm] = fab1(arr)
            for r, nm in enumerate(LM_NAMES):
                local[nm] = fab1(cs["lm"][r])
                local[nm + "_temp"] = fab1(np.zeros((nz, ny, nx)))
            for nm in ("rho_tgt_temp", "u_tgt_temp", "v_tgt_temp", "w_tgt_temp", "temp_tgt_temp"):
                local[nm] = fab1(np.zeros((nz, ny, nx)))
            fs = cs["fs_uvwT"]
            g.update(fs_u=fs[0], fs_v=fs[1], fs_w=fs[2], temperature=fs[3])
            for nm, v in zip(("su_chi", "su_zeta_x", "su_zeta_y", "su_zeta_z", "su_pixx", "su_piyy", "su_pizz",
                              "su_pixy", "su_pixz", "su_piyz", "su_lambda_x", "su_lambda_y", "su_lambda_z"),
                             cs["su_lm"]):
                g[nm] = float(v)
            self.set_step(cs.get("step", 0))
        local.update(lvl=F.FInt(0), dummy_fout=0.0, dummy_gout=0.0,
                     wax_lo=F.FArray(np.array([0, 0, 0], np.int64), [1]),
                     wax_hi=F.FArray(np.array([nx - 1, ny - 1, nz - 1], np.int64), [1]),
                     state=F.FArray(fab(st, -666, np.int64), lb),
                     fout=F.FArray(fab(cs["fout"], 0.0, np.float64), lb),
                     gout=F.FArray(fab(cs["gout"], 0.0, np.float64), lb),
                     fi=F.FArray(fab(cs["prev_f"], 0.0, np.float64), lb),
                     gi=F.FArray(fab(cs["prev_g"], 0.0, np.float64), lb),
                     node_pt=F.FArray(np.zeros((nx + 2 * G, ny + 2 * G, nz + 2 * G, 1), np.int64), lb))
        local["fine"] = F.FInt(0)
        self.procs["lu_decomp"] = self.real_lu  # (the recording wrapper caps its log at 200 updates)
        try:
            self.interp.run([reach_if, kg_stmt, loop], local, scope)
        finally:
            self.procs["lu_decomp"] = self._lu_hook

        def valid(name):
            return np.ascontiguousarray(np.transpose(local[name].a[G:G + nx, G:G + ny, G:G + nz, :], (3, 2, 1, 0)))

        return valid("fi"), valid("gi"), int(local["reach"])

    def explode(self, root, f, g, crs_lm, crs_rho, crs_temp, step):
        """interlevel_interpolation.f95's per-node block for one fine ghost node (state
        1e7..1.1e9): the coarse multipliers, the interpolated f and g (each negative or NaN
        pair replaced by the coarse equilibrium), the moments, the multiplier solve from the
        coarse multipliers and alpha.  Returns f, g, the 13 multipliers, rho, u, v, w, T, alpha."""
        lines = F.logical_lines((root / "looping/timestepping/interlevel/interlevel_interpolation.f95").read_text())
        k_if = next(k for k, (no, s) in enumerate(lines)
                    if re.match(r"^if \(state\(a,b,c,1\) >=\s*10000000 \.and\.", s))
        block, _ = F.parse_stmt(lines, k_if)
        local = {}
        scope = self.interp.scope_for(local)
        self.interp.declare("integer :: a,b,c,i,lvl", local, scope, set())
        self.interp.declare("real(kind=dp) :: rho_sum,u_sum,v_sum,w_sum,energy_sum,v_mag,pxx,pyy,pzz,pxy,pxz,pyz,"
                            "mu_c,mu_f,kappa_c,kappa_f,old_fi(dir),fieq_skip(dir),loc_fi_diff(dir)", local, scope,
                            set())
        node = lambda vals, dt=np.float64: F.FArray(np.asarray(vals, dt).reshape(1, 1, 1, -1).copy(), [1, 1, 1, 1])  # noqa: E731
        one = lambda v: node([v])  # noqa: E731
        nan = float("nan")
        local.update(a=F.FInt(1), b=F.FInt(1), c=F.FInt(1), lvl=F.FInt(0), valid_interp_nodes=False,
                     state=node([10000001] * 39, np.int64), fi=node(np.full(39, nan)), gi=node(np.full(39, nan)),
                     crs_fi=node(f), crs_gi=node(g), crs_rho=one(crs_rho), crs_temp=one(crs_temp),
                     rho=one(crs_rho), u_vel=one(nan), v_vel=one(nan), w_vel=one(nan), temp=one(crs_temp),
                     alpha=one(nan))
        for r, nm in enumerate(LM_NAMES):
            local["crs_" + nm] = one(crs_lm[r])
            local[nm] = one(nan)
        self.set_step(step)
        self.procs["lu_decomp"] = self.real_lu
        try:
            self.interp.run([block], local, scope)
        finally:
            self.procs["lu_decomp"] = self._lu_hook
        v = lambda nm: local[nm].a.ravel().tolist()  # noqa: E731
        return {"f": v("fi"), "g": v("gi"), "lm": [local[nm].a.ravel()[0] for nm in LM_NAMES],
                "m5": [v(nm)[0] for nm in ("rho", "u_vel", "v_vel", "w_vel", "temp")], "alpha": v("alpha")[0]}

    def ggm_box(self, root, q, u, v, w, state, scheme, limit, q_fs, G=8):
        """calculate_grad_mag.f95's and calculate_gradgrad_mag.f95's loops over one box (tux_lo
        = 0; PGS off): q (the variable), u, v, w and the 39 link codes of the box; its FABs get G
        ghost layers holding q_fs, zero velocities and node type -666.  scheme 0 central,
        1 upwind, 2 downwind.  Returns gm, ggm and the tags (nz, ny, nx) of the box."""
        out = {}
        for fname in ("calculate_grad_mag.f95", "calculate_gradgrad_mag.f95"):
            lines = F.logical_lines((root / "GGM/derivatives" / fname).read_text())
            k = next(k for k, (no, s) in enumerate(lines) if re.match(r"^do c = tux_lo\(3\)", s))
            out[fname] = F.parse_stmt(lines, k)[0]
            if fname.startswith("calculate_grad_mag"):
                k_r = next(k for k, (no, s) in enumerate(lines) if s.startswith("reach = "))
                out["reach"] = F.parse_stmt(lines, k_r)[0]
        nz, ny, nx = q.shape

        def fab(arr, fill, dtype=np.float64, comps=1):
            o = np.full((nx + 2 * G, ny + 2 * G, nz + 2 * G, comps), fill, dtype)
            t = np.transpose(arr, tuple(range(arr.ndim))[::-1])
            o[G:G + nx, G:G + ny, G:G + nz, :] = t.reshape(nx, ny, nz, comps)
            return F.FArray(o, [-G, -G, -G, 1])

        local = {}
        scope = self.interp.scope_for(local)
        self.interp.declare("integer :: a,b,c,reach", local, scope, set())
        self.interp.declare("real(kind=dp) :: x_der,y_der,z_der", local, scope, set())
        tags = np.full((nx, ny, nz), "0", object)
        local.update(g=F.FInt(1), lvl=F.FInt(0), settag="1", cleartag="0",
                     tux_lo=F.FArray(np.array([0, 0, 0], np.int64)),
                     tux_hi=F.FArray(np.array([nx - 1, ny - 1, nz - 1], np.int64)),
                     tagarr=F.FArray(tags, [0, 0, 0]), state=fab(state, -666, np.int64, 39),
                     holder=fab(q, q_fs), gm=fab(np.zeros_like(q), 0.0), ggm=fab(np.zeros_like(q), 0.0),
                     u_vel=fab(u, 0.0), v_vel=fab(v, 0.0), w_vel=fab(w, 0.0))
        self.g.update(upwind=scheme == 1, downwind=scheme == 2, central=scheme == 0, nghosts=F.FInt(6),
                      ggm_tag_limit=F.FArray(np.array([limit]), [0]), use_pgs=False)
        self.interp.run([out["reach"], out["calculate_grad_mag.f95"], out["calculate_gradgrad_mag.f95"]], local, scope)

        def valid(nm):
            return np.ascontiguousarray(np.transpose(local[nm].a[G:G + nx, G:G + ny, G:G + nz, 0], (2, 1, 0)))

        return valid("gm"), valid("ggm"), np.transpose(tags == "1", (2, 1, 0)).astype(np.uint8)

    def pgs(self, root, ggm, u, v, w, s0, sensitivity, max_scan, G=8):
        """GGM/PGS/predictive_splitter.f95's loop over one box (tux_lo = 0): ggm, u, v, w and
        the node types s0 (nz, ny, nx) of the box; its FABs get G ghost layers of node type -666
        (which no scan counts) and ggm 0.  Returns the tags (nz, ny, nx), 1 where set."""
        lines = F.logical_lines((root / "GGM/PGS/predictive_splitter.f95").read_text())
        k_loop = next(k for k, (no, s) in enumerate(lines) if re.match(r"^do c = tux_lo\(3\),tux_hi\(3\)$", s))
        loop, _ = F.parse_stmt(lines, k_loop)
        nz, ny, nx = s0.shape

        def fab(arr, fill, dtype=np.float64, comps=1):
            out = np.full((nx + 2 * G, ny + 2 * G, nz + 2 * G, comps), fill, dtype)
            out[G:G + nx, G:G + ny, G:G + nz, 0] = np.transpose(arr, (2, 1, 0))
            return F.FArray(out, [-G, -G, -G, 1])

        local = {}
        scope = self.interp.scope_for(local)
        self.interp.declare("integer :: a,b,c,x,y,z,v,reach(6)", local, scope, set())
        self.interp.declare("logical :: x_upwind,y_upwind,z_upwind,u_dominant,v_dominant,w_dominant,victory",
                            local, scope, set())
        tags = np.full((nx, ny, nz), "0", object)
        st = fab(s0, -666, np.int64, 39)
        local.update(g=F.FInt(1), settag="1", cleartag="0", pgs_limit=2 * sensitivity, pgs_upper=3 * sensitivity,
                     tux_lo=F.FArray(np.array([0, 0, 0], np.int64)),
                     tux_hi=F.FArray(np.array([nx - 1, ny - 1, nz - 1], np.int64)),
                     tagarr=F.FArray(tags, [0, 0, 0]), state=st, ggm=fab(ggm, 0.0),
                     u_vel=fab(u, 0.0), v_vel=fab(v, 0.0), w_vel=fab(w, 0.0))
        self.g.update(pgs_max_scan=F.FInt(max_scan), ggm_sensitivity=sensitivity, nghosts=F.FInt(G))
        self.interp.run([loop], local, scope)
        return np.transpose(tags == "1", (2, 1, 0)).astype(np.uint8)

    def shifted_ibb(self, i, code_i, fieq_opp, gieq_opp, rho, tgt, ul, vl, wl, Tl, sp):
        """shifted_ibb.f95 for wall link i (1-based) of a node: its code of direction i, the
        equilibria of the closure's direction, rho, the (u, v, w, T) targets, the seven-point
        stencil's u, v, w, T and node types; returns (fout, gout)."""
        v = {"fo": float("nan"), "go": float("nan")}
        node = F.FArray(np.full((1, 1, 1, 39), -1, np.int64), [1, 1, 1, 1])
        node.set((1, 1, 1, i), code_i)
        vec = lambda vals, dt=np.float64: F.FArray(np.asarray(vals, dt).copy())  # noqa: E731
        nan = float("nan")
        self.interp.call("shifted_ibb", [F.Ref(v, "fo"), nan, nan, nan, float(fieq_opp), nan, nan, F.Ref(v, "go"),
                                         nan, nan, nan, float(gieq_opp)] + [float(x) for x in tgt] +
                         [F.FInt(i), F.FInt(0), node, float(rho), vec(ul), vec(vl), vec(wl), vec(Tl),
                          vec(sp, np.int64), F.FInt(0), F.FInt(1), F.FInt(1), F.FInt(1)])
        return v["fo"], v["go"]

    def targets(self, code, up, vp, wp, Tp, fi):
        """target_finder.f95 for one node (a = b = c = 1): its 39 link codes, u, v, w, T at
        x + c_j, and its post-streaming slots; returns rho, u, v, w, T targets."""
        out = {n: float("nan") for n in ("r", "u", "v", "w", "t")}
        node = lambda vals, dt=np.float64: F.FArray(np.asarray(vals, dt).reshape(1, 1, 1, 39), [1, 1, 1, 1])  # noqa: E731
        vec = lambda vals: F.FArray(np.asarray(vals, np.float64).copy())  # noqa: E731
        self.interp.call("target_finder", [node(code, np.int64), vec(up), vec(vp), vec(wp), vec(Tp), node(fi)] +
                         [F.Ref(out, n) for n in ("r", "u", "v", "w", "t")] + [F.FInt(1), F.FInt(1), F.FInt(1)])
        return [out[n] for n in ("r", "u", "v", "w", "t")]

    def damp(self, root, fout, gout, state, fs_f, fs_g, lo, hi, ng=8):
        """damp_it.f95 on one box at level 0: its reach, then its in-place sweep (direction
        outermost) over the box and `reach` ghost layers.  fout, gout, state: (39, nz, ny, nx)
        of the box; their FABs get ng ghost layers holding fs_f, fs_g (the freestream
        equilibria, positive) and the node code -666 in every component (outside an
        external-flow domain); fi and gi are positive everywhere, so the sweep's parts for
        them leave them alone.  The
        box's bounds, a derived type there, are passed as the arrays fux_lo, fux_hi.
        nghosts_mid is 8: directions_and_weights.f95 sets it (:355-362) before it sets
        shifted (:479), so the module's initial .false. picks the unshifted value."""
        lines = [(no, s.replace("fux%lo(", "fux_lo(").replace("fux%hi(", "fux_hi("))
                 for no, s in F.logical_lines((root / "looping/timestepping/damp_it.f95").read_text())]
        k_reach = next(k for k, (no, s) in enumerate(lines) if s == "if (.not. shifted) then")
        k_loop = next(k for k, (no, s) in enumerate(lines) if re.match(r"^do\s+i\s*=\s*1\s*,\s*dir$", s))
        reach_if, _ = F.parse_stmt(lines, k_reach)
        loop, _ = F.parse_stmt(lines, k_loop)
        nz, ny, nx = fout.shape[1:]

        def fab_of(pop, fs):
            fab = np.empty((nx + 2 * ng, ny + 2 * ng, nz + 2 * ng, 39))
            fab[...] = np.asarray(fs)[None, None, None, :]
            fab[ng:ng + nx, ng:ng + ny, ng:ng + nz, :] = np.transpose(pop, (3, 2, 1, 0))
            return fab

        ffab, gfab = fab_of(fout, fs_f), fab_of(gout, fs_g)
        sfab = np.full((nx + 2 * ng, ny + 2 * ng, nz + 2 * ng, 39), -666, np.int64)
        sfab[ng:ng + nx, ng:ng + ny, ng:ng + nz, :] = np.transpose(state, (3, 2, 1, 0))
        lb = [lo[0] - ng, lo[1] - ng, lo[2] - ng, 1]
        local = {}
        scope = self.interp.scope_for(local)
        self.interp.declare("integer :: a,b,c,i,reach", local, scope, set())
        self.g["nghosts_mid"] = F.FInt(8)
        # the sweep also repairs fi (the post-streaming populations, which the next streaming
        # overwrites except in slots no rule writes); positive here, so that part does nothing
        local.update(lvl=F.FInt(0), fout=F.FArray(ffab, lb), gout=F.FArray(gfab, lb), state=F.FArray(sfab, lb),
                     fi=F.FArray(np.ones_like(ffab), lb), gi=F.FArray(np.ones_like(gfab), lb),
                     fux_lo=F.FArray(np.array(lo, np.int64), [1]), fux_hi=F.FArray(np.array(hi, np.int64), [1]))
        self.interp.run([reach_if, loop], local, scope)

        def valid(name):
            out = local[name].a[ng:ng + nx, ng:ng + ny, ng:ng + nz, :]
            return np.ascontiguousarray(np.transpose(out, (3, 2, 1, 0)))

        return valid("fout"), valid("gout"), int(local["reach"])

    def collide(self, root, f, g, lm, rho, u, v, w, T, alpha):
        """The body of collision.f95's per-node loop for one node (a = b = c = 1)."""
        lines = F.logical_lines((root / "looping/timestepping/collision.f95").read_text())
        i0 = next(k for k, (no, s) in enumerate(lines) if re.match(r"^if\s*\(state\(a,b,c,1\)\s*<\s*0\)\s*cycle", s))
        body, _ = F.parse_block(lines, i0, r"^end\s*do")
        k_lead = next(k for k, (no, s) in enumerate(lines) if s.startswith("lead_gieq_const"))
        # the routine's declarations, then its set-up statement lead_gieq_const = 2 C_v - D (collision.f95:73)
        local = {}
        scope = self.interp.scope_for(local)
        for no, s in lines[1:k_lead]:
            if F._DECL.match(s):
                self.interp.declare(s, local, scope, set())
        for name in ("loc_fieq", "loc_gieq", "loc_fi_diff", "q_bar_dir", "contr_heat_flux", "loc_gi_diff",
                     "old_fout"):
            local[name] = F.FArray(np.full(39, np.nan))
        self.interp.run([F.parse_stmt(lines, k_lead)[0]], local, scope)

        def node_arr(vals):
            a = np.asarray(vals, np.float64).reshape(1, 1, 1, -1)
            return F.FArray(a.copy(), [1, 1, 1, 1])

        local.update(a=F.FInt(1), b=F.FInt(1), c=F.FInt(1), lvl=F.FInt(0),
                     state=F.FArray(np.zeros((1, 1, 1, 39), np.int64), [1, 1, 1, 1]),
                     fi=node_arr(f), gi=node_arr(g), fout=node_arr(np.full(39, np.nan)),
                     gout=node_arr(np.full(39, np.nan)), rho=node_arr([rho]), u_vel=node_arr([u]),
                     v_vel=node_arr([v]), w_vel=node_arr([w]), temp=node_arr([T]), alpha=node_arr([alpha]))
        for n, x in zip(LM_NAMES, lm):
            local[n] = node_arr([x])
        try:
            self.interp.run(body, local, scope)
        except F._Cycle:
            raise RuntimeError("the node was skipped")
        return local["fout"].a.ravel().tolist(), local["gout"].a.ravel().tolist()


def case_consts(s39, shifted: bool):
    if shifted:
        c = s39.wedge_case_consts()
    else:
        c = s39.wedge_case_consts(v_inf_ms=0.5 * math.sqrt(1.4 * s39.GAS_CONST_R * 288.15), use_shifted=False)
    # a Knudsen-scale epsilon large enough that the heat-flux corrections show in every population
    c.elbm_epsilon = 0.37
    return c


def main(root: pathlib.Path) -> None:
    s39 = _setup_module()
    rng = np.random.default_rng(20241204)
    rng_w = np.random.default_rng(20241205)  # the stored (previous-step) w of the flow-variable cases
    out = {"lattices": {}}
    damp_out = {}
    for shifted in (True, False):
        c = case_consts(s39, shifted)
        ref = Reference(root, c, shifted)
        lat = {"consts": {k: getattr(c, k) for k in CONST_FIELDS}, "su_lm": list(c.su_lm),
               "tables": ref.tables(), "cases": []}
        lat["consts"]["shifted"] = int(shifted)
        # target_finder on seeded nodes: wall links (packed distances) among interior, null and
        # boundary links, the fields at x + c_j and the node's slots
        rng_t = np.random.RandomState(4242 + int(shifted))
        tcases = []
        for _ in range(8):
            code = rng_t.choice([0, 0, 3, -10, -666, -1000], 39).astype(np.int64)
            walls = rng_t.random_sample(39) < 0.3
            walls[rng_t.randint(1, 39)] = True
            code[walls] = -1001 - np.floor(rng_t.uniform(0.02, 0.98, int(walls.sum())) * 1e9).astype(np.int64)
            up, vp, wp = (c.mach * rng_t.uniform(-1.2, 1.2, 39) for _ in range(3))
            Tp = c.temperature * rng_t.uniform(0.8, 1.2, 39)
            fi_n = rng_t.uniform(0.001, 0.2, 39)
            tcases.append({"code": code.tolist(), "u": up.tolist(), "v": vp.tolist(), "w": wp.tolist(), "T": Tp.tolist(),
                           "fi": fi_n.tolist(), "fs_temp": c.temperature,
                           "out": ref.targets(code, up, vp, wp, Tp, fi_n)})
        lat["targets"] = tcases
        # calculate_alpha across its branches: deviations from equilibrium scaled from tiny (alpha =
        # 2 below the chi_3 threshold) to large (the quadratic root clamped to [alpha_sum_min, 2.125])
        rng_a = np.random.RandomState(6060 + int(shifted))
        lm_fs = s39.freestream_start_lm(c)
        _, fe_a, _ = ref.lagrange(1.0, c.mach, 0.0, 0.0, c.temperature,
                                  [c.temperature + c.mach ** 2, c.temperature, c.temperature, 0.0, 0.0, 0.0], lm_fs)
        acases = []
        for scale in (1e-12, 1e-6, 1e-3, 0.02, 0.1, 0.3, 0.6, 0.9):
            for step in (3, c.startup_timesteps + 5):
                fd = np.asarray(fe_a) * scale * rng_a.uniform(-1, 1, 39)
                f = (np.asarray(fe_a) - fd).tolist()
                ref.set_step(step)
                a = ref.alpha(f, fd.tolist(), c.temperature)
                acases.append({"f": f, "fd": fd.tolist(), "T": c.temperature, "step": step, "alpha": a})
        lat["alpha_branches"] = acases
        # interlevel_interpolation.f95's per-node explosion on seeded interpolants (some with a
        # negative f and a NaN g, which take the coarse equilibrium)
        rng_e = np.random.RandomState(99 + int(shifted))
        lm_fs = s39.freestream_start_lm(c)
        ecases = []
        for n_case in range(6):
            rho0, u0 = 1.0 + 0.02 * rng_e.uniform(-1, 1), c.mach * (1 + 0.05 * rng_e.uniform(-1, 1))
            T0 = c.temperature * (1 + 0.02 * rng_e.uniform(-1, 1))
            P0 = [rho0 * (T0 + u0 * u0), rho0 * T0 + 1e-4, rho0 * T0 - 1e-4, 1e-4, -1e-4, 0.0]
            lm_c, fe, _ = ref.lagrange(rho0, u0, 0.01, -0.01, T0, P0, lm_fs)
            lead = 2.0 * c.const_vol - 3
            f = np.asarray(fe) * (1 + 0.03 * rng_e.uniform(-1, 1, 39))
            g = lead * T0 * np.asarray(fe) * (1 + 0.03 * rng_e.uniform(-1, 1, 39))
            if n_case >= 3:
                f[rng_e.randint(0, 39)] = -0.01
                g[rng_e.randint(0, 39)] = float("nan")
            crs_rho, crs_T = rho0 * (1 + 0.01 * rng_e.uniform(-1, 1)), T0 * (1 + 0.01 * rng_e.uniform(-1, 1))
            step = 3 if n_case % 2 == 0 else c.startup_timesteps + 30
            r = ref.explode(root, f, g, lm_c, crs_rho, crs_T, step)
            ecases.append({"f": [x if math.isfinite(x) else None for x in f.tolist()],
                           "g": [x if math.isfinite(x) else None for x in g.tolist()], "lm": list(lm_c),
                           "rho": crs_rho, "T": crs_T, "step": step, "out": r})
        lat["explode"] = ecases
        if shifted:
            # shifted_ibb on seeded wall links: stencil node types interior, solid (-1001) or
            # null (-666), before and after the start-up ramps
            rng_s = np.random.RandomState(5151)
            scases = []
            for n_case in range(16):
                i = int(rng_s.randint(1, 40))
                code_i = int(-1001 - np.floor(rng_s.uniform(0.02, 0.98) * 1e9))
                sp = [0] + rng_s.choice([0, 0, 0, -1001, -666, -1001 - 400000000], 6).tolist()
                tgt = [c.mach * rng_s.uniform(0.0, 1.0), c.mach * rng_s.uniform(-0.2, 0.2),
                       c.mach * rng_s.uniform(-0.2, 0.2), c.temperature * rng_s.uniform(0.9, 1.3)]
                ul, vl, wl = (c.mach * rng_s.uniform(-0.3, 1.2, 7) for _ in range(3))
                Tl = c.temperature * rng_s.uniform(0.8, 1.4, 7)
                rho = float(rng_s.uniform(0.8, 1.3))
                fe, ge = float(rng_s.uniform(0.001, 0.1)), float(rng_s.uniform(0.001, 0.1))
                step = 3 if n_case % 2 == 0 else c.startup_timesteps + 11
                ref.set_step(step)
                fo, go = ref.shifted_ibb(i, code_i, fe, ge, rho, tgt, ul, vl, wl, Tl, sp)
                scases.append({"i": i, "code": code_i, "fieq": fe, "gieq": ge, "rho": rho, "tgt": tgt,
                               "u": ul.tolist(), "v": vl.tolist(), "w": wl.tolist(), "T": Tl.tolist(), "sp": sp,
                               "step": step, "fout": fo, "gout": go})
            lat["shifted_ibb"] = scases
        lm_start = s39.freestream_start_lm(c)
        for k in range(3):
            rho = float(rng.uniform(0.92, 1.08))
            u = float(c.mach * rng.uniform(0.9, 1.1))
            v, w = (float(x) for x in rng.uniform(-0.25, 0.25, 2))
            T = float(c.temperature * rng.uniform(0.95, 1.05))
            P = [rho * (T + u * u) * rng.uniform(0.995, 1.005), rho * (T + v * v) * rng.uniform(0.995, 1.005),
                 rho * (T + w * w) * rng.uniform(0.995, 1.005), rho * u * v + rng.uniform(-1e-3, 1e-3),
                 rho * u * w + rng.uniform(-1e-3, 1e-3), rho * v * w + rng.uniform(-1e-3, 1e-3)]
            P = [float(x) for x in P]
            lm, fe, lus = ref.lagrange(rho, u, v, w, T, P, lm_start)
            expo0 = ref.fieq(rho, lus[0]["lm_in"])
            # a non-equilibrium node around the solved equilibrium
            f = (np.asarray(fe) * (1.0 + rng.uniform(-0.03, 0.03, 39))).tolist()
            lead = 2.0 * c.const_vol - 3
            g = (lead * T * np.asarray(fe) * (1.0 + rng.uniform(-0.03, 0.03, 39))).tolist()
            fd = (np.asarray(fe) - np.asarray(f)).tolist()
            gd = (lead * T * np.asarray(fe) - np.asarray(g)).tolist()
            w_old = float(w + rng_w.uniform(-0.05, 0.05))
            flow = {"w_old": w_old, "out": ref.flow_vars(root, f, g, w_old)}
            steps = {}
            for step in (3, c.startup_timesteps + 7):
                ref.set_step(step)
                a = ref.alpha(f, fd, T)
                fo, go = ref.collide(root, f, g, lm, rho, u, v, w, T, a)
                steps[str(step)] = {"alpha": a, "q_bar": ref.q_bar(fd, fe, u, v, w, T),
                                    "little_q_bar": ref.little_q_bar(gd, u, v, w, T), "fout": fo, "gout": go}
            lat["cases"].append({
                "rho": rho, "u": u, "v": v, "w": w, "T": T, "P": P, "lm0": list(lm_start),
                "lm": lm, "fieq": fe, "iterations": len(lus), "expo0": expo0, "lu": lus[:2],
                "f": f, "g": g, "fd": fd, "gd": gd, "flow": flow, "steps": steps})
        out["lattices"]["shifted" if shifted else "unshifted"] = lat
        # the fout repair of a box with link codes
        def changes(before, after):
            k = np.flatnonzero(after.ravel() != before.ravel())
            return [[int(j), float(after.ravel()[j])] for j in k]

        for name, (sh, *_) in damp39_inputs.CASES.items():
            if sh != shifted:
                continue
            fo, go, st, fs_f, fs_g = damp39_inputs.case(name)
            lo, hi = damp39_inputs.bounds(name)
            rf, rg, reach = ref.damp(root, fo, go, st, fs_f, fs_g, lo, hi)
            damp_out[name] = {"consts": lat["consts"], "lo": list(lo), "hi": list(hi), "reach": reach,
                              "negative_f": int((fo < 0).sum()), "negative_g": int((go < 0).sum()),
                              "changed_f": changes(fo, rf), "changed_g": changes(go, rg)}
    # lu_decomp on dense, diagonally dominant matrices, where both index quirks change the result at O(1)
    recs = []
    for k in range(4):
        J = rng.uniform(-1.0, 1.0, (13, 13)) + np.eye(13) * 6.0
        moments = [float(x) for x in rng.uniform(-1.0, 1.0, 13)]
        lm = {n: float(x) for n, x in zip(LM_NAMES, rng.uniform(-1.0, 1.0, 13))}
        lm_in = [lm[n] for n in LM_NAMES]
        md = {"v": 0.0}
        jac = F.FArray(J.copy())
        ref.interp.call_proc(ref.real_lu, [jac, F.FInt(13)] + moments + [F.Ref(lm, n) for n in LM_NAMES] +
                             [F.Ref(md, "v")])
        recs.append({"jacobian": J.ravel().tolist(), "moments": moments, "lm_in": lm_in,
                     "lm_out": [lm[n] for n in LM_NAMES], "max_diff": md["v"]})
    out["lu_dense"] = recs
    # derivative_windage_secondord (the GGM derivative), every combination of its four link
    # states, the three schemes and both wind signs
    wrec = []
    for scheme in range(3):
        up, down, cen = scheme == 1, scheme == 2, scheme == 0
        for bits in range(16):
            for wind in (0.37, -0.29):
                q = [float(x) for x in rng.uniform(-1.0, 1.0, 5)]
                st5 = [0] + [0 if (bits >> b) & 1 else -10 for b in range(4)]
                dq = ref.interp.call("derivative_windage_secondord",
                                     [F.FArray(np.array(q)), F.FArray(np.array(st5, np.int64)), wind, up, down, cen])
                wrec.append({"scheme": scheme, "q": q, "state": st5, "wind": wind, "dq": float(dq)})
    out["windage"] = wrec
    # predictive splitting over a box
    ggm, u, v, w, s0 = pgs_inputs.case()
    tags = ref.pgs(root, ggm, u, v, w, s0, pgs_inputs.SENSITIVITY, pgs_inputs.MAX_SCAN)
    out["pgs"] = {"tagged": np.flatnonzero(tags.ravel()).tolist()}
    # the gradient magnitudes and the tags of calculate_grad_mag / calculate_gradgrad_mag: gm at
    # every node of the box, ggm and the tags where the +-2 stencil stays inside it (the ghost
    # nodes' gm, which the reference computes from the ghost layers, is left out)
    gcases = []
    for scheme in range(3):
        rho, u, v, w, state, rho_fs = pgs_inputs.ggm_case(scheme)
        gm, ggm, gtags = ref.ggm_box(root, rho, u, v, w, state, scheme, 0.05, rho_fs)
        inner = np.zeros(rho.shape, bool)
        inner[2:-2, 2:-2, 2:-2] = True
        gcases.append({"scheme": scheme, "limit": 0.05, "gm": push39_inputs.digest(gm),
                       "ggm_inner": push39_inputs.digest(ggm[inner]),
                       "tagged_inner": np.flatnonzero(gtags[inner]).tolist()})
    out["ggm"] = gcases
    (HERE / "d3q39_core_golden.json").write_text(json.dumps(out))
    (HERE / "d3q39_damp_golden.json").write_text(json.dumps(damp_out))
    push_out = {}
    for name, (sh, *_) in push39_inputs.CASES.items():
        c = case_consts(s39, bool(sh))
        ref = Reference(root, c, bool(sh))
        cs = push39_inputs.case(name, s39)
        fi, gi, reach = ref.push(root, cs)
        fluid = cs["state"][0] >= 0
        push_out[name] = {"consts": {k: getattr(c, k) for k in CONST_FIELDS}, "reach": reach,
                          "fluid_nodes": int(fluid.sum()), "fi": push39_inputs.digest(fi[:, fluid]),
                          "gi": push39_inputs.digest(gi[:, fluid])}
        push_out[name]["consts"]["shifted"] = int(sh)
    wall_cases = [(name, s39.wedge_case_consts(), push39_inputs.wall_case(name, s39))
                  for name in push39_inputs.WALL_CASES]
    wall_cases.append(("unshifted_walls",) + push39_inputs.unshifted_wall_case(s39))
    for name, c, cs in wall_cases:
        sh = bool(cs["shifted"])
        ref = Reference(root, c, sh)
        fi, gi, reach = ref.push(root, cs)
        fluid = cs["state"][0] >= 0
        wall = (cs["state"] <= -1001) & fluid[None]
        wall[0] = False
        # the slots a wall closure's value can reach: slot opp(i) of wall link i, and slot i where a
        # later bounce-back of link opp(i) writes it from the rewritten fout(x, i)
        opp = s39.lattice39(int(sh), 1)[3]
        wall = wall | wall[opp]
        other = fluid[None] & ~wall
        push_out[name] = {"consts": {k: getattr(c, k) for k in CONST_FIELDS}, "reach": reach,
                          "fluid_nodes": int(fluid.sum()), "wall_slots": int(wall.sum()),
                          "fi": push39_inputs.digest(fi[other]), "gi": push39_inputs.digest(gi[other]),
                          "fi_wall": fi[wall].tolist(), "gi_wall": gi[wall].tolist()}
        push_out[name]["consts"]["shifted"] = int(sh)
    (HERE / "d3q39_push_golden.json").write_text(json.dumps(push_out, indent=0))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_d3q39_core_golden.py <reference root>")
    main(pathlib.Path(sys.argv[1]))
