"""The oracle (a NumPy restatement of the reference) against golden vectors
produced by running the reference itself (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from conftest import golden, rel_l2
from oracle import spectral as O
from phrike_gb300 import problems

TAGS = ["d1f0", "d1f1", "d0f0", "d0f1"]


@pytest.mark.parametrize("tag", TAGS)
def test_operators_match_reference(tag):
    ops = golden("fourier_ops.npz")
    d, f = bool(int(tag[1])), bool(int(tag[3]))
    b1 = O.FourierBox((64,), (1.0,), dealias=d, filter_enabled=f)
    x = ops[f"g1_{tag}_in"]
    assert rel_l2(b1.deriv(x, 0), ops[f"g1_{tag}_dx"]) < 1e-13
    assert rel_l2(b1.filt(x), ops[f"g1_{tag}_filt"]) < 1e-13
    b2 = O.FourierBox((16, 32), (0.5, 1.0), dealias=d, filter_enabled=f)
    x = ops[f"g2_{tag}_in"]
    assert rel_l2(b2.deriv(x, 1), ops[f"g2_{tag}_dx"]) < 1e-13
    assert rel_l2(b2.deriv(x, 0), ops[f"g2_{tag}_dy"]) < 1e-13
    assert rel_l2(b2.filt(x), ops[f"g2_{tag}_filt"]) < 1e-13
    b3 = O.FourierBox((16, 8, 16), (4 * np.pi, np.pi, 2 * np.pi), dealias=d, filter_enabled=f)
    x = ops[f"g3_{tag}_in"]
    assert rel_l2(b3.deriv(x, 2), ops[f"g3_{tag}_dx"]) < 1e-13
    assert rel_l2(b3.deriv(x, 1), ops[f"g3_{tag}_dy"]) < 1e-13
    assert rel_l2(b3.deriv(x, 0), ops[f"g3_{tag}_dz"]) < 1e-13
    assert rel_l2(b3.filt(x), ops[f"g3_{tag}_filt"]) < 1e-13


@pytest.mark.parametrize("N", [128, 1024])
def test_sod_steps_match_reference(N):
    z = golden(f"sod1d_n{N}.npz")
    U0 = problems.sod_smoothed(N)
    np.testing.assert_array_equal(U0, z["U0"])
    s = O.EulerSolver(O.FourierBox((N,), (1.0,), dealias=True, filter_enabled=True))
    assert rel_l2(s.rhs(U0), z["rhs0"]) < 1e-13
    U = U0
    for _ in range(int(z["nsteps"])):
        U = s.step(U, float(z["dt"]))
    for c in range(3):
        assert rel_l2(U[c], z["U"][c]) < 1e-12
    assert abs(s.compute_dt(U0) - float(z["dt_cfl0"])) < 1e-15
    cons = O.conserved_sums(U, 1.4)
    np.testing.assert_allclose([cons["mass"], cons["momentum"], cons["energy"]], z["cons"], rtol=1e-12)


@pytest.mark.parametrize("shape,nsteps", [((16, 16, 16), 3), ((32, 8, 16), 2)])
def test_tgv_steps_match_reference(shape, nsteps):
    Nz, Ny, Nx = shape
    z = golden(f"tgv3d_{Nx}x{Ny}x{Nz}.npz")
    U0 = problems.taylor_green_3d(Nx, Ny, Nz)
    np.testing.assert_array_equal(U0, z["U0"])
    s = O.EulerSolver(O.FourierBox(shape, (2 * np.pi,) * 3, dealias=True), cfl=0.25)
    assert rel_l2(s.rhs(U0), z["rhs0"]) < 1e-13
    U = U0
    for _ in range(nsteps):
        U = s.step(U, 1e-3)
    for c in range(5):
        assert rel_l2(U[c], z["U"][c]) < 1e-12
    assert abs(O.max_wave_speed(U0, 1.4) - float(z["speed0"])) < 1e-12


@pytest.mark.parametrize("nx,ny", [(32, 32), (64, 16)])
def test_khi_cfl_run_matches_reference(nx, ny):
    z = golden(f"khi2d_{nx}x{ny}.npz")
    U0 = problems.kelvin_helmholtz_2d(nx, ny, U0=float(z["U0_param"]), A=float(z["A"]))
    np.testing.assert_array_equal(U0, z["U0"])
    s = O.EulerSolver(O.FourierBox((ny, nx), (1.0, 1.0), dealias=True), cfl=0.4)
    assert rel_l2(s.rhs(U0), z["rhs0"]) < 1e-13
    U, t, dts = s.run(U0, 0.0, 1.0, max_steps=len(z["dts"]))
    np.testing.assert_allclose(dts, z["dts"], rtol=1e-13)
    for c in range(4):
        assert rel_l2(U[c], z["U"][c]) < 1e-12


def test_separable_rewrite_is_exact():
    """The pass decomposition D_x P_y P_z used by the CUDA kernels equals the
    reference's full N-D transform (up to rounding) for every mask/filter
    combination, including the Nyquist term with dealiasing off."""
    rng = np.random.default_rng(5)
    for d in (True, False):
        for f in (True, False):
            box = O.FourierBox((8, 16, 32), (1.0, 2.0, 3.0), dealias=d, filter_enabled=f)
            x = rng.standard_normal((8, 16, 32))
            for a in range(3):
                y = x
                for b in range(3):
                    one = O.FourierBox((box.shape[b],), (box.lengths[b],), dealias=d, filter_enabled=f)
                    y = np.moveaxis(y, b, -1)
                    y = one.deriv(y, 0) if a == b else one.filt(y)
                    y = np.moveaxis(y, -1, b)
                assert rel_l2(y, box.deriv(x, a)) < 1e-12


@pytest.mark.parametrize("nx,ny", [(17, 17), (33, 17)])
def test_lgl_oracle_matches_reference(nx, ny):
    """LGL x LGL acoustic pulse with walls: nodes, D matrices, the rhs (with
    walls applied first), steps and the CFL dt against the reference's torch
    float64 backend."""
    from oracle import lgl as L
    z = golden(f"lgl2d_{nx}x{ny}.npz")
    s = L.LGLSolver2D(nx, ny, 2.0, 2.0, gamma=1.4)
    np.testing.assert_allclose(s.ax.x, z["x"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(s.ay.x, z["y"], rtol=0, atol=1e-14)
    assert np.abs(s.ax.D - z["Dx"]).max() <= 1e-12 * np.abs(z["Dx"]).max()
    assert np.abs(s.ay.D - z["Dy"]).max() <= 1e-12 * np.abs(z["Dy"]).max()
    U0 = problems.acoustic_pulse_lgl_2d(z["x"] - 1.0, z["y"] - 1.0, gamma=1.4, amp=float(z["amp"]),
                                        width2=float(z["width2"]))
    np.testing.assert_allclose(U0, z["U0"], rtol=0, atol=1e-15)
    assert rel_l2(s.rhs(U0.copy()), z["rhs0"]) < 1e-12
    U = U0.copy()
    for _ in range(int(z["nsteps"])):
        U = s.step(U, float(z["dt"]))
    for c in range(4):
        assert rel_l2(U[c], z["U"][c]) < 1e-13, c
    assert abs(s.compute_dt(U0) - float(z["dt_cfl0"])) <= 1e-14 * float(z["dt_cfl0"])


@pytest.mark.parametrize("tag", ["wall", "mixed"])
def test_lgl1d_oracle_matches_reference(tag):
    """1D Legendre grid: nodes, the rhs with the boundary codes applied first,
    five steps (RK4 with the filter at cadence 2; RK2 with a per-boundary,
    per-variable bc map and gravity) and the CFL dt against the reference."""
    from lgl1d_cases import CASES, DT, LENGTH, NSTEPS, initial_state
    from oracle import lgl as L
    c = CASES[tag]
    z = golden("lgl1d.npz")
    s = L.LGLSolver1D(c["n"], LENGTH, gamma=1.4, filter_params=c["filter_params"], cfl=0.4,
                      bc=c["bc"] if c["bc"] is not None else "dirichlet", gravity=c["gravity"], scheme=c["scheme"])
    np.testing.assert_allclose(s.ax.x, z[f"{tag}_x"], rtol=0, atol=1e-14)
    U0 = initial_state(s.ax.x)
    np.testing.assert_allclose(U0, z[f"{tag}_U0"], rtol=0, atol=1e-14)
    assert rel_l2(s.rhs(U0.copy()), z[f"{tag}_rhs0"]) < 1e-12
    U = U0.copy()
    for _ in range(NSTEPS):
        U = s.step(U, DT)
    for k in range(3):
        assert rel_l2(U[k], z[f"{tag}_U"][k]) < 1e-13, k
    assert abs(s.compute_dt(U0) - float(z[f"{tag}_dt0"])) <= 1e-13 * float(z[f"{tag}_dt0"])


def test_lgl1d_bc_codes():
    """Boundary resolution: walls zero the momentum and copy the rest; a
    per-boundary map with a bare string applies to every variable."""
    from oracle import lgl as L
    np.testing.assert_array_equal(L.bc_codes_1d("dirichlet"), [[L.BC_COPY, L.BC_ZERO, L.BC_COPY]] * 2)
    np.testing.assert_array_equal(L.bc_codes_1d("open"), [[L.BC_COPY] * 3] * 2)
    np.testing.assert_array_equal(L.bc_codes_1d({"left": "wall", "right": {"rho": "neumann", "u": "periodic"}}),
                                  [[L.BC_COPY, L.BC_ZERO, L.BC_COPY], [L.BC_COPY, L.BC_NONE, L.BC_COPY]])


@pytest.mark.parametrize("bc", [None, "wall", "reflective", "neumann", "open", "periodic",
                                {"density": "open", "momentum": "dirichlet"},
                                {"x0": "open", "x_max": {"pressure": "periodic", "mom": "open"}}])
def test_lgl1d_grid_bc_codes_match_oracle(bc):
    """The grid's boundary resolver (host code handed to the plan descriptor)
    agrees with the oracle's for every form of the configuration."""
    from oracle import lgl as L
    from phrike_gb300.grid import _bc_codes_1d
    want = L.bc_codes_1d(bc if bc is not None else "dirichlet").reshape(-1).tolist()
    assert _bc_codes_1d(bc if bc is not None else "dirichlet") == want


def test_lgl_filter_preserves_low_modes():
    """The nodal filter keeps constants and linear functions (sigma_0 = 1,
    sigma_1 = exp(-alpha/(n-1)^p) ~ 1) and damps the top mode by e^-alpha."""
    from oracle import lgl as L
    ax = L.LGLAxis(33, 2.0)
    F = ax.nodal_filter(8, 36.0)
    one = np.ones(33)
    np.testing.assert_allclose(F @ one, one, atol=1e-13)
    top = ax.V[:, -1]
    assert np.linalg.norm(F @ top) < 1e-14 * np.linalg.norm(top) + np.exp(-36.0) * np.linalg.norm(top) * 2


@pytest.mark.parametrize("nx,ny", [(32, 32), (32, 16)])
def test_mhd_oracle_matches_reference(nx, ny):
    """2D ideal MHD (Orszag-Tang plus a divergent B perturbation): rhs,
    projection, steps (filter on / off), CFL dt, conserved sums and div B
    against the reference's NumPy path."""
    from oracle import mhd as M
    z = golden(f"mhd2d_{nx}x{ny}.npz")
    fp = {"enabled": True, "p": 8, "alpha": 36.0} if int(z["filter"]) else None
    s = M.MHDSolver2D(nx, ny, filter_params=fp, cfl=0.3)
    U0 = z["U0"]
    ref = problems.orszag_tang_2d(nx, ny, gamma=5.0 / 3.0)
    np.testing.assert_allclose(U0[:5], ref[:5], rtol=0, atol=1e-12)  # only B was perturbed
    rhs = s.rhs(U0)
    for c in range(8):
        assert rel_l2(rhs[c], z["rhs0"][c]) < 1e-12, c
    P = s.project(U0)
    for c in range(8):
        assert rel_l2(P[c], z["P0"][c]) < 1e-12, c
    assert s.max_div_b(P) < 1e-12 and s.max_div_b(U0) > 1e-2
    U = U0.copy()
    for _ in range(int(z["nsteps"])):
        U = s.step(U, float(z["dt"]))
    for c in range(8):
        assert rel_l2(U[c], z["U"][c]) < 1e-12, c
    assert abs(s.compute_dt(U0) - float(z["dt_cfl0"])) < 1e-14
    cons = M.conserved_quantities(U0, 5.0 / 3.0)
    np.testing.assert_allclose(list(cons.values()), z["cons0"], rtol=1e-12, atol=1e-12)


def test_gravity_and_artificial_viscosity_match_reference():
    """Constant gravity (2D KHI, 3D TGV) and artificial viscosity (1D Sod in
    sensor mode with its default filter cadence 5; 2D KHI in sensor mode on
    the 'pressure' variable, which the reference's 2D sensor reads as u_y, and
    in constant mode) against the reference's NumPy path."""
    z = golden("sources.npz")
    s = O.EulerSolver(O.FourierBox((32, 32), (1.0, 1.0), dealias=True), gravity=[0.3, -1.0])
    assert rel_l2(s.rhs(z["grav2d_U0"]), z["grav2d_rhs0"]) < 1e-13
    U = z["grav2d_U0"].copy()
    for _ in range(3):
        U = s.step(U, 2e-3)
    assert rel_l2(U, z["grav2d_U"]) < 1e-13
    s3 = O.EulerSolver(O.FourierBox((16, 16, 16), (2 * np.pi,) * 3, dealias=True), gravity=[0.2, -0.5, 1.0])
    assert rel_l2(s3.rhs(z["grav3d_U0"]), z["grav3d_rhs0"]) < 1e-13
    T = z["grav3d_U0"].copy()
    for _ in range(2):
        T = s3.step(T, 1e-3)
    assert rel_l2(T, z["grav3d_U"]) < 1e-13
    av = {"enabled": True, "mode": "sensor", "nu_max": 2e-3, "s_ref": 1.0, "s_min": 0.1, "p": 2.0,
          "epsilon": 1e-12, "sensor_variable": "density"}
    assert int(z["av1d_interval"]) == 5
    s1 = O.EulerSolver(O.FourierBox((128,), (1.0,), dealias=True, filter_enabled=True), av=av, filter_interval=5)
    assert rel_l2(s1.rhs(z["av1d_U0"]), z["av1d_rhs0"]) < 1e-13
    S = z["av1d_U0"].copy()
    for _ in range(7):
        S = s1.step(S, 2e-5)
    assert rel_l2(S, z["av1d_U"]) < 1e-13
    for mode, cfg in (("sensor", dict(av, sensor_variable="pressure")),
                      ("constant", {"enabled": True, "mode": "constant", "nu_constant": 1e-3})):
        s2 = O.EulerSolver(O.FourierBox((32, 32), (1.0, 1.0), dealias=True), av=cfg)
        assert rel_l2(s2.rhs(z["grav2d_U0"]), z[f"av2d_{mode}_rhs0"]) < 1e-13, mode
        V = z["grav2d_U0"].copy()
        for _ in range(3):
            V = s2.step(V, 2e-3)
        assert rel_l2(V, z[f"av2d_{mode}_U"]) < 1e-13, mode


@pytest.mark.parametrize("tag", ["sod_rk45", "sod_rk23_tight", "sod_av_grav_rk45", "khi_rk23", "tgv_rk78",
                                 "ot_rk45"])
def test_adaptive_rk_matches_reference(tag):
    """Embedded RK23 / RK45 / the reference's 8-stage "rk78" with its step
    controller, rejections and forced acceptance, through the reference's run
    loops (1D with viscosity and gravity; 2D with gravity; 3D; 2D MHD)."""
    from adaptive_cases import accepted_steps, run_oracle
    z = golden("adaptive.npz")
    U, t, log, _, _ = run_oracle(tag, z[f"{tag}_U0"])
    ref = z[f"{tag}_steps"]
    got = accepted_steps(log)
    assert got.shape == ref.shape, (got.shape, ref.shape)
    np.testing.assert_array_equal(got[:, 0], ref[:, 0])
    np.testing.assert_allclose(got[:, 1], ref[:, 1], rtol=1e-9)
    assert abs(t - float(z[f"{tag}_t"])) < 1e-12
    assert rel_l2(U, z[f"{tag}_U"]) < 1e-10
    if tag == "sod_rk23_tight":  # rejections and forced acceptances both occur
        assert len(log) > len(got)


def test_rk2_scheme_matches_reference():
    """scheme="rk2" (midpoint) fixed steps of the 1D (filter cadence 2), 2D,
    3D and MHD solvers against the reference's own runs."""
    from oracle import mhd as M
    z = golden("rk2.npz")
    fbox = dict(dealias=True, filter_enabled=True)
    s1 = O.EulerSolver(O.FourierBox((128,), (1.0,), **fbox), filter_interval=2, scheme="rk2")
    U = z["sod_U0"].copy()
    for _ in range(5):
        U = s1.step(U, 2e-4)
    assert rel_l2(U, z["sod_U"]) < 1e-13
    s2 = O.EulerSolver(O.FourierBox((32, 32), (1.0, 1.0), **fbox), scheme="rk2")
    V = z["khi_U0"].copy()
    for _ in range(4):
        V = s2.step(V, 1e-3)
    assert rel_l2(V, z["khi_U"]) < 1e-13
    s3 = O.EulerSolver(O.FourierBox((16, 16, 16), (2 * np.pi,) * 3, dealias=True), cfl=0.25, scheme="rk2")
    T = z["tgv_U0"].copy()
    for _ in range(3):
        T = s3.step(T, 1e-3)
    assert rel_l2(T, z["tgv_U"]) < 1e-13
    sm = M.MHDSolver2D(32, 32, filter_params={"enabled": True, "p": 8, "alpha": 36.0}, scheme="rk2")
    W = z["ot_U0"].copy()
    for _ in range(3):
        W = sm.step(W, 2e-3)
    assert rel_l2(W, z["ot_U"]) < 1e-12


def test_mhd_resistivity_viscosity_match_reference():
    """2D MHD with explicit resistivity and viscosity (the spectral Laplacian
    with mask and filter, Nyquist modes included when dealiasing is off) and
    the parabolic CFL limit, against the reference's own runs."""
    from oracle import mhd as M
    z = golden("mhd_diffusion.npz")
    for tag, (nx, ny), fp, dealias, eta, nu in (("a", (32, 32), {"enabled": True, "p": 8, "alpha": 36.0}, True,
                                                  0.02, 0.01),
                                                 ("b", (32, 16), None, False, 0.2, 0.0)):
        s = M.MHDSolver2D(nx, ny, filter_params=fp, dealias=dealias, cfl=0.3, resistivity=eta, viscosity=nu,
                          cfl_diff=0.8)
        U0 = z[f"{tag}_U0"]
        assert rel_l2(s.rhs(U0), z[f"{tag}_rhs0"]) < 1e-12, tag
        assert abs(s.compute_dt(U0) - float(z[f"{tag}_dt"])) < 1e-12 * float(z[f"{tag}_dt"]), tag
        U = U0.copy()
        for _ in range(3):
            U = s.step(U, 1e-3)
        assert rel_l2(U, z[f"{tag}_U"]) < 1e-12, tag


def test_mhd1d_matches_reference():
    """1D MHD (SpectralSolverMHD1D): right-hand side, the 1D projection
    (Bx -> mean, thermal pressure held), ideal RK4 and resistive/viscous RK2
    steps, the CFL dt with the exact fast speed and the parabolic limit, and
    the CFL run, against the reference."""
    from oracle import mhd as M
    z = golden("mhd1d.npz")
    fp = {"enabled": True, "p": 8, "alpha": 36.0}
    U0 = z["U0"]
    for tag, kw, scheme in (("ideal", {}, "rk4"), ("diff", {"resistivity": 0.01, "viscosity": 0.005}, "rk2")):
        s = M.MHDSolver1D(128, 1.0, filter_params=fp, cfl=0.4, scheme=scheme, **kw)
        assert rel_l2(s.rhs(U0), z[f"{tag}_rhs0"]) < 1e-12, tag
        assert rel_l2(s.project(U0), z[f"{tag}_P0"]) < 1e-14, tag
        assert abs(s.compute_dt(U0) - float(z[f"{tag}_dt0"])) < 1e-12 * float(z[f"{tag}_dt0"]), tag
        U = U0.copy()
        for _ in range(4):
            U = s.step(U, 1e-3)
        assert rel_l2(U, z[f"{tag}_U"]) < 1e-12, tag
    s = M.MHDSolver1D(128, 1.0, filter_params=fp, cfl=0.4)
    U = s.project(U0)
    t, dts = 0.0, []
    while t < 0.05 - 1e-12:
        dt = min(s.compute_dt(U), 0.05 - t)
        U = s.step(U, dt)
        t += dt
        dts.append(dt)
    np.testing.assert_allclose(dts, z["cfl_dts"], rtol=1e-12)
    assert rel_l2(U, z["cfl_U"]) < 1e-12


@pytest.mark.parametrize("name", ["d1", "d1_nyq", "d2", "d2_nyq", "d3", "d3_nyq"])
def test_tracer_oracle_matches_reference(name):
    """Point evaluation of a random field and of the velocity, and tracer
    positions after leap-frog steps, against the reference's grids and
    tracer classes (dealias on with the filter, and off: Nyquist modes)."""
    import tracer_cases as TC
    from oracle import tracers as OT
    z = golden("tracers.npz")
    shape, lengths, dealias, filt, _ = TC.CASES[name]
    lxyz = list(reversed(lengths))
    pos = TC.tracer_positions(name)
    f = OT.eval_points(TC.field(name), pos, lxyz, dealias, filt)
    assert np.abs(f - z[f"{name}_f"]).max() <= 1e-12 * np.abs(z[f"{name}_f"]).max()
    U = TC.state(name)
    tr = OT.Tracers(*pos)
    v = tr.velocity(U, lxyz, dealias, filt)
    assert np.abs(v - z[f"{name}_vel"]).max() <= 1e-12 * np.abs(z[f"{name}_vel"]).max()
    for _ in range(TC.STEPS):
        tr.step(U, TC.DT, lxyz, dealias, filt)
    assert np.abs(np.stack(tr.pos) - z[f"{name}_pos"]).max() < 1e-13


def test_tracer_config_layouts():
    """tracers_from_config draws the reference's seeded random and uniform
    layouts (problems/base.py:961-1021), without a device."""
    from phrike_gb300.tracers import tracers_from_config

    class G:  # a stand-in 3D Fourier grid: only shape and lengths are read
        _shape, _basis, Lx, Ly, Lz = (4, 4, 4), "fourier", 1.0, 2.0, 3.0

    t = tracers_from_config(G, {"enabled": True, "num": 5, "seed": 42})
    rng = np.random.default_rng(42)
    want = [rng.uniform(0.0, L, size=5) for L in (1.0, 2.0, 3.0)]
    np.testing.assert_array_equal(np.stack([t.x, t.y, t.z]), np.stack(want))
    u = tracers_from_config(G, {"enabled": True, "num": 8, "layout": "uniform"})
    assert len(u.x) == 8 and float(np.max(u.z)) < 3.0
    assert tracers_from_config(G, {"enabled": False}) is None


@pytest.mark.parametrize("name", ["alfven", "turb"])
def test_mhd3d_oracle_matches_reference(name):
    """3D MHD: rhs (with resistivity and viscosity in the turb case), the
    projected state, fixed-dt steps (RK4 with the filter; RK2), the CFL dt,
    div B and the conserved sums against SpectralSolverMHD3D."""
    import mhd3d_cases as MC
    from oracle import mhd as M
    z = golden("mhd3d.npz")
    nx, ny, nz, lx, ly, lz, filt, cfg, scheme, dt, nsteps = MC.CASES[name]
    s = M.MHDSolver3D(nx, ny, nz, lx, ly, lz, gamma=MC.GAMMA, filter_params=filt, cfl=0.3, scheme=scheme,
                      resistivity=cfg.get("resistivity", 0.0), viscosity=cfg.get("viscosity", 0.0))
    U0 = MC.initial_state(name)
    np.testing.assert_allclose(U0, z[f"{name}_U0"], rtol=0, atol=1e-15)
    assert rel_l2(s.rhs(U0.copy()), z[f"{name}_rhs0"]) < 1e-12
    assert rel_l2(s.project(U0.copy()), z[f"{name}_P0"]) < 1e-13
    U = U0.copy()
    for _ in range(nsteps):
        U = s.step(U, dt)
    for c in range(8):
        assert rel_l2(U[c], z[f"{name}_U"][c]) < 1e-12 or np.abs(U[c] - z[f"{name}_U"][c]).max() < 1e-13, c
    assert abs(s.compute_dt(U0) - float(z[f"{name}_dt0"])) <= 1e-13 * float(z[f"{name}_dt0"])
    assert s.max_div_b(U) < 1e-12
    cons = M.conserved_quantities(U, MC.GAMMA)
    np.testing.assert_allclose([cons[k] for k in ("mass", "momentum_x", "momentum_y", "momentum_z", "energy",
                                                  "magnetic_energy", "cross_helicity")], z[f"{name}_cons"],
                               rtol=1e-12, atol=1e-10)


@pytest.mark.parametrize("shape", [(64,), (32, 16), (16, 8, 32)])
def test_fused_oracle_matches_per_derivative_oracle(shape):
    """The large-grid oracle form (one spectral sum per stage, real
    transforms) against the per-derivative full transforms the reference
    uses, on right-hand sides and three RK4 steps."""
    nd = len(shape)
    if nd == 1:
        U0 = problems.sod_smoothed(shape[0])
        box = lambda: O.FourierBox(shape, (1.0,), dealias=True, filter_enabled=True)
    elif nd == 2:
        U0 = problems.kelvin_helmholtz_2d(shape[1], shape[0], U0=1.2, A=0.02)
        box = lambda: O.FourierBox(shape, (1.0, 1.0), dealias=True)
    else:
        U0 = problems.taylor_green_3d(shape[2], shape[1], shape[0])
        box = lambda: O.FourierBox(shape, (2 * np.pi,) * 3, dealias=True)
    a, f = O.EulerSolver(box()), O.EulerSolver(box(), fused=True)
    assert rel_l2(f.rhs(U0), a.rhs(U0)) < 1e-12
    Ua, Uf = U0, U0
    for _ in range(3):
        Ua, Uf = a.step(Ua, 1e-4), f.step(Uf, 1e-4)
    for c in range(len(U0)):
        assert np.abs(Uf[c] - Ua[c]).max() <= 1e-12 * np.abs(Ua).max()
