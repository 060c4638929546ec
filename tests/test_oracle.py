"""The CPU oracle against known answers and its committed golden fixtures.

No golden outputs exist for the reference (it ships no tests and no model
outputs) and it cannot be compiled here (no Fortran compiler), so the oracle
is pinned by known-answer tests that follow from the reference's algorithm:
the van Leer limiter, linear dispersion, the Poisson coefficients of a flat
bed, a lake at rest staying at rest (well-balanced bed-slope source,
src/source_terms.F:447-453), mass growing by exactly (ALPHA(3)+BETA(3)) per
SSP-RK3 step (1/3 and 2/3 are default-real literals, src/initialize.F:3386-3391),
and mirror symmetry.
"""
import math
import os

import numpy as np
import pytest

from conftest import rel_l2

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = {"tiny_c1": 6, "tiny_c2": 6, "tiny_c3": 6, "tiny_c4": 4}


def golden_path(name, steps):
    return os.path.join(HERE, "golden", f"{name}_{steps}steps.npz")


def test_limiter_known_values(oracle_mod):
    L = oracle_mod.limiter
    assert L(1.0, 1.0) == 1.0
    assert L(1.0, -1.0) == 0.0
    assert L(2.0, 1.0) == pytest.approx(4.0 / 3.0, rel=1e-15)   # 2ab/(a+b)
    assert L(-3.0, -1.0) == pytest.approx(-1.5, rel=1e-15)


def test_wave_dispersion(oracle_mod):
    from nhwave_gb300 import scenarios as S
    p, d, e, u = S.make("tiny_c2")
    o = oracle_mod.Oracle(p, d, e, u)
    sigma = 2.0 * math.pi / 2.02
    k = o.params and oracle_mod.lib().orc_wave_number(o._h, sigma)
    g = float(np.float32(9.81))
    assert sigma ** 2 == pytest.approx(g * k * math.tanh(k * 0.4), rel=1e-7)


def test_flat_bed_poisson_coefficients(oracle_mod):
    from nhwave_gb300 import default_params
    M, N, K = 4, 3, 3
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=0.5, dy=0.25, tol=1e-12)
    depth = np.full(M * N, 2.0)
    o = oracle_mod.Oracle(p, depth)
    oracle_mod.lib().orc_generate_coef_rhs(o._h)
    coef, rhs = o.coef_rhs()
    ds = float(np.float32(1.0) / np.float32(K))
    a1 = 1.0 / 4.0                       # DelzS^2 with D = 2, flat bed, eta = 0
    ic = 1 + M * (1 + N * 1)             # interior point, away from every boundary
    assert coef[0, ic] == pytest.approx(2 / 0.25 + 2 / 0.0625 + 2 * a1 / ds ** 2, rel=1e-14)
    assert coef[5, ic] == pytest.approx(-a1 / ds ** 2, rel=1e-14)
    assert coef[12, ic] == pytest.approx(-a1 / ds ** 2, rel=1e-14)
    assert coef[1, ic] == coef[8, ic] == -1 / 0.25
    assert np.all(coef[[3, 4, 6, 7, 10, 11, 13, 14], ic] == 0.0)  # no slope terms on a flat bed
    assert np.all(rhs == 0.0)                                        # fluid at rest
    top = 1 + M * (1 + N * (K - 1))
    assert np.all(coef[[3, 4, 5, 6, 7], top] == 0.0)                 # Dirichlet P = 0 above


@pytest.mark.parametrize("hllc", [0, 1])
def test_lake_at_rest(hllc, oracle_mod):
    """A lake at rest stays at rest but for the SSP-RK3 coefficient sum: each step
    scales D by ALPHA(3)+BETA(3) = 1 + 2.98e-8, lifting eta by Hc*(g^n - 1)."""
    from nhwave_gb300 import default_params, fields as F
    rng = np.random.default_rng(3)
    M, N, K = 24, 10, 4
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=1.0, dy=1.0, tol=1e-12, dt_ini=0.05, hllc=hllc)
    depth = 5.0 + rng.uniform(0.0, 2.0, size=M * N)
    o = oracle_mod.Oracle(p, depth)
    n = 4
    for _ in range(n):
        assert o.step() == 0
    sl = o.shape.interior
    g = float(np.float32(1.0) / np.float32(3.0)) + float(np.float32(2.0) / np.float32(3.0))
    hc = depth.reshape(N, M)
    eta = o.get(F.ETA)[sl(F.ETA)]
    lift = hc * (g ** n - 1.0)
    # the non-uniform lift itself drives a flow of the same tiny order
    assert np.abs(eta - lift).max() < 0.2 * lift.max()
    assert np.abs(o.get(F.U)[sl(F.U)]).max() < 1e-6


@pytest.mark.parametrize("hllc", [0, 1])
def test_mass_grows_by_rk_coefficient_sum(hllc, oracle_mod):
    from nhwave_gb300 import scenarios as S
    p, d, e, u = S.make("tiny_c1", hllc=hllc)
    p.tol = 1e-12
    o = oracle_mod.Oracle(p, d, e, u)
    m0 = o.mass()
    n = 5
    for _ in range(n):
        assert o.step() == 0
    growth = float(np.float32(1.0) / np.float32(3.0)) + float(np.float32(2.0) / np.float32(3.0))
    assert o.mass() / m0 == pytest.approx(growth ** n, abs=1e-13)


@pytest.mark.parametrize("hllc", [0, 1])
def test_mirror_symmetry(hllc, oracle_mod):
    from nhwave_gb300 import default_params, fields as F
    M, N, K = 30, 6, 4
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=0.5, dy=0.5, tol=1e-13, dt_ini=0.01, hllc=hllc)
    x = (np.arange(M) + 0.5) * 0.5
    eta = 0.05 * np.exp(-((x - 7.5) / 2.0) ** 2)
    o = oracle_mod.Oracle(p, np.full(M * N, 2.0), np.tile(eta, N))
    for _ in range(4):
        assert o.step() == 0
    e2 = o.get(F.ETA)[o.shape.interior(F.ETA)]
    # HLLC's left mass flux is DUxL + SxL*(DxL*(SxL-UxL)/(SxL-SxS) - DxL)
    # (src/nhwave.F:1792, 2585, 2799): at SxS = 0 it is DUxL - DxL*UxL, the
    # gap between the reconstructed D*U and the product of the reconstructed
    # D and U, and the right one is its mirror image.  The branch SxS >= 0
    # takes the left one, so on the symmetry plane (SxS = 0) the mass flux is
    # that second-order gap instead of zero: the mirror image holds to
    # O(dx^2 * slope products) only
    lim = 1e-12 if not hllc else 1e-6
    assert np.abs(e2 - e2[:, ::-1]).max() < lim * np.abs(e2).max()


def test_hllc_close_to_hll_on_a_smooth_wave(oracle_mod):
    """HLLC (src/nhwave.F:2555-2670) differs from HLL only by the contact
    wave's star state: on a smooth, subcritical wave both agree to the
    truncation error, the mass is the same to rounding, and they differ."""
    from nhwave_gb300 import fields as F, scenarios as S
    out = []
    for hllc in (0, 1):
        p, d, e, u = S.make("tiny_c2", hllc=hllc)
        p.tol = 1e-12
        o = oracle_mod.Oracle(p, d, e, u)
        for _ in range(6):
            assert o.step() == 0
        out.append((o.get(F.ETA)[o.shape.interior(F.ETA)], o.mass()))
    r = rel_l2(out[1][0], out[0][0])
    assert 0.0 < r < 1e-2
    assert out[1][1] == pytest.approx(out[0][1], rel=1e-13)


@pytest.mark.parametrize("name", list(GOLDEN))
def test_oracle_reproduces_golden(name, oracle_mod):
    from nhwave_gb300 import fields as F, scenarios as S
    steps = GOLDEN[name]
    ref = np.load(golden_path(name, steps))
    p, d, e, u = S.make(name, seed=7)
    p.tol = 1e-14
    p.itmax = 5000
    o = oracle_mod.Oracle(p, d, e, u)
    for _ in range(steps):
        assert o.step() == 0
    for f in ("ETA", "D", "U", "V", "W", "P", "OMEGA"):
        fid = getattr(F, f)
        assert rel_l2(o.get(fid)[o.shape.interior(fid)], ref[f]) < 1e-12, f
    assert np.array_equal(o.get(F.MASK)[o.shape.interior(F.MASK)], ref["MASK"])
    s = o.scalars()
    assert s.time == pytest.approx(ref["scalars"][0], rel=1e-14)


def test_wet_dry_front_exists_in_slide_case(oracle_mod):
    ref = np.load(golden_path("tiny_c3", GOLDEN["tiny_c3"]))
    mask = ref["MASK"]
    assert 0 < (mask == 0).sum() < mask.size


def test_flume_linear_inflow_follows_the_boundary_wave(oracle_mod):
    """LEF_LIN through BC_X0 = 3 (src/waves.F:808-855): eta in the first
    interior column follows the imposed boundary elevation 0.5*A*sin(sigma t)."""
    import math
    from nhwave_gb300 import fields as F, scenarios as S
    p, d, e, u = S.make("tiny_flume_lin")
    p.tol, p.itmax = 1e-10, 5000
    o = oracle_mod.Oracle(p, d, e, u)
    ts, e0 = [], []
    for _ in range(150):
        assert o.step() == 0
        ts.append(o.scalars().time)
        e0.append(o.get(F.ETA)[o.shape.interior(F.ETA)][:, 0].mean())
    ts, e0 = np.array(ts), np.array(e0)
    ref = 0.5 * p.amp_wave * np.sin(2 * math.pi / p.per_wave * ts)
    assert np.corrcoef(e0, ref)[0, 1] > 0.97
    assert 0.85 < e0.std() / ref.std() < 1.1


def test_flume_solitary_inflow_arrives_with_its_height(oracle_mod):
    """LEF_SOL (src/waves.F:869-903): the boundary elevation peaks at about
    the wave height when the crest, started 4h/sqrt(A/h) upstream, arrives."""
    import math
    from nhwave_gb300 import fields as F, scenarios as S
    p, d, e, u = S.make("tiny_flume_sol")
    p.tol, p.itmax = 1e-10, 5000
    o = oracle_mod.Oracle(p, d, e, u)
    A, h = p.amp_wave, p.dep_wave
    arrival = 4 * h / math.sqrt(A / h) / math.sqrt(9.81 * h * (1 + A / h))
    peak, t_peak = 0.0, 0.0
    while o.scalars().time < arrival + 0.5:
        assert o.step() == 0
        v = o.get(F.ETA)[o.shape.interior(F.ETA)][:, 0].mean()
        if v > peak:
            peak, t_peak = v, o.scalars().time
    assert abs(peak - A) < 0.15 * A
    assert abs(t_peak - arrival) < 0.15


def test_statistics_of_a_lake_at_rest(oracle_mod):
    """statistics (src/nhwave.F:3118-3160) of a flat lake: with eta = 0 and
    uniform sigma levels the potential energy from z = 0 is
    -Rho0 g dx dy sum D^2 * sum_k dsig_k (1 - sigc_k) = -Rho0 g dx dy sum D^2 / 2,
    the kinetic energy is zero, and MassVolume is sum D dx dy."""
    from nhwave_gb300 import default_params
    rng = np.random.default_rng(4)
    M, N, K = 12, 7, 5
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=0.5, dy=0.25, tol=1e-12, dt_ini=0.05)
    depth = 2.0 + rng.uniform(0.0, 1.0, size=M * N)
    o = oracle_mod.Oracle(p, depth)
    st = o.statistics()
    g = float(np.float32(9.81))
    assert st["mass_volume"] == pytest.approx(depth.sum() * 0.5 * 0.25, rel=1e-14)
    assert st["energy"] == pytest.approx(-0.5 * 1000.0 * g * 0.5 * 0.25 * (depth ** 2).sum(), rel=1e-6)
    assert st["max_eta"] == 0.0 and st["min_eta"] == 0.0
    assert st["max_u"] == st["max_v"] == st["max_w"] == 0.0


def test_orlanski_east_side_lets_a_solitary_wave_out(oracle_mod):
    """BC_Xn = 6 (Orlanski radiation, src/nhwave.F:4599-4621 and 5197-5206):
    a solitary wave running into the east side leaves through it.  After the
    crest reaches the side (t > 3 s) a wall reflects it at full height; the
    open side keeps well under that (the radiation speed is estimated from
    the last two steps' values, so part of the wave still comes back), and
    water leaves the domain."""
    from nhwave_gb300 import fields as F, scenarios as S

    def run(bc_xn):
        p, d, e, u = S.solitary_channel(M=80, N=3, K=4, dx=0.1, h=0.5, amp=0.05, x0=4.0, bc_xn=bc_xn)
        p.tol, p.itmax = 1e-8, 5000
        o = oracle_mod.Oracle(p, d, e, u)
        m0, late = o.mass(), 0.0
        while o.scalars().time < 4.0:
            assert o.step() == 0
            if o.scalars().time > 3.0:
                late = max(late, np.abs(o.get(F.ETA)[o.shape.interior(F.ETA)]).max())
        return late, o.mass() / m0

    wall, wall_mass = run(1)
    open_, open_mass = run(6)
    assert wall > 0.9 * 0.05
    assert open_ < 0.75 * wall
    assert wall_mass == pytest.approx(1.0, abs=1e-4)
    assert open_mass < wall_mass - 1e-3


def _west_boundary_eta(o):
    """Ein_X0 recovered from the west ghost column: wl_bc sets D there to
    2 Din - D(Ibeg), so on a flat bed the mean of eta over the first ghost and
    first interior column is Ein (row-averaged over the interior rows)."""
    from nhwave_gb300 import fields as F
    e = o.get(F.ETA)
    return 0.5 * (e[2:-2, 1] + e[2:-2, 2]).mean()


def test_elliptic_functions_against_scipy(oracle_mod):
    """cnoidal_cn / cnoidal_ck / cnoidal_ce (src/waves.F:225-370) against
    scipy's Jacobi cn and complete elliptic integrals (parameter m).  K and E
    carry the single-precision pi literal of the reference (2.8e-8 relative)."""
    sp = pytest.importorskip("scipy.special")
    L = oracle_mod.lib()
    for m in (0.1, 0.5, 0.9135, 0.999, 1.0 - 1e-8):
        K, E = L.orc_elliptic(1, 0.0, m), L.orc_elliptic(2, 0.0, m)
        assert K == pytest.approx(sp.ellipk(m), rel=1e-7), m
        assert E == pytest.approx(sp.ellipe(m), rel=1e-7), m
        for u in (0.0, 0.3, 1.1, -2.0, 0.5 * K, K):
            assert L.orc_elliptic(0, u, m) == pytest.approx(sp.ellipj(u, m)[1], abs=1e-12), (u, m)


def test_cnoidal_wave_parameters(oracle_mod):
    """cnoidal (src/waves.F:184-220) for H = 0.1 m, h = 0.5 m, T = 3 s: the
    trough level makes the mean elevation over a wave length zero, and the
    length is the period times the celerity of the reference's formula."""
    import ctypes
    sp = pytest.importorskip("scipy.special")
    out = (ctypes.c_double * 3)()
    H, h, T = 0.1, 0.5, 3.0
    assert oracle_mod.lib().orc_cnoidal_wave(H, h, T, out) == 0
    L, yt, m = out
    assert 0.85 < m < 0.95 and -H < yt < 0
    K, E = sp.ellipk(m), sp.ellipe(m)
    u = np.linspace(0.0, 2 * K, 20001)[:-1]
    assert abs((yt + H * sp.ellipj(u, m)[1] ** 2).mean()) < 1e-6 * H
    g = float(np.float32(9.81))
    c = math.sqrt(g * h * (1.0 + H / h / m * (-m + 2.0 - 3.0 * E / K)))
    assert L == pytest.approx(c * T, rel=0.02)
    assert oracle_mod.lib().orc_cnoidal_wave(0.02, 0.5, 1.5, out) != 0   # deep water: m leaves (0, 1]


def test_flume_cnoidal_inflow_over_one_period(oracle_mod):
    """LEF_CON (src/waves.F:92-170): the boundary elevation starts at its
    zero crossing and over one period spans the wave height, trough to
    crest, with zero mean."""
    from nhwave_gb300 import scenarios as S
    p, d, e, u = S.make("tiny_flume_con")
    p.tol, p.itmax = 1e-8, 5000
    o = oracle_mod.Oracle(p, d, e, u)
    ts, ein = [], []
    while o.scalars().time < p.per_wave:
        assert o.step() == 0
        ts.append(o.scalars().time)
        ein.append(_west_boundary_eta(o))
    ts, ein = np.array(ts), np.array(ein)
    H = p.amp_wave
    assert abs(ein[0]) < 0.1 * H
    assert (ein.max() - ein.min()) == pytest.approx(H, rel=0.02)
    w = np.gradient(ts)
    assert abs((ein * w).sum() / w.sum()) < 0.03 * H


def test_flume_stokes_inflow_follows_the_formula(oracle_mod):
    """LEF_STK (src/waves.F:518-560): the boundary elevation is the
    second-order Stokes wave 0.5 A cos(phi) + A^2 k/16 cosh(kh)/sinh^3(kh)
    (2 + cosh 2kh) cos(2 phi), phi = pi/2 - sigma t."""
    from nhwave_gb300 import scenarios as S
    p, d, e, u = S.make("tiny_flume_stk")
    p.tol, p.itmax = 1e-8, 5000
    o = oracle_mod.Oracle(p, d, e, u)
    pi = float(np.float32(3.141592653))
    sigma = 2.0 * pi / p.per_wave
    k = oracle_mod.lib().orc_wave_number(o._h, sigma)
    h, A = p.dep_wave, p.amp_wave
    e2 = A * A * k / 16.0 * math.cosh(k * h) / math.sinh(k * h) ** 3 * (2.0 + math.cosh(2.0 * k * h))
    for _ in range(40):
        assert o.step() == 0
        ph = pi / 2 - sigma * o.scalars().time
        assert _west_boundary_eta(o) == pytest.approx(0.5 * A * math.cos(ph) + e2 * math.cos(2 * ph), abs=1e-12)


def _viscous_channel(oracle_mod, M, N, K, u_profile, T, **kw):
    """Flat 1 m deep channel started from a velocity profile U (K, N); runs to
    time T and returns (time, U interior (K, N, M))."""
    from nhwave_gb300 import default_params, fields as F
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=0.2, dy=0.2, dt_ini=0.01, dt_max=0.02, tol=1e-10,
                       itmax=2000, viscous_flow=1, visc=1e-6, **kw)
    uvw = np.zeros((3, K, N, M))
    uvw[0] = u_profile[:, :, None]
    o = oracle_mod.Oracle(p, np.ones(M * N), None, uvw.ravel())
    while o.scalars().time < T:
        assert o.step() == 0
    return o.scalars().time, o.get(F.U)[o.shape.interior(F.U)]


def test_viscous_vertical_mode_decays_at_the_diffusion_rate(oracle_mod):
    """Implicit vertical viscous step (src/nhwave.F:690-1182, trig :13182-13224)
    with IVTURB = 1: a depth-mean-free shear U = U0 cos(pi sigma) in a flat
    channel decays as exp(-nu lambda t), lambda = (2 - 2 cos(pi/K)) / (D dsig)^2
    the discrete Neumann eigenvalue, nu = VISCOSITY + Cvs / Schmidt."""
    K = 10
    sig = (np.arange(K) + 0.5) / K
    prof = 0.01 * np.cos(np.pi * sig)[:, None] * np.ones((1, 3))
    t, u = _viscous_channel(oracle_mod, 80, 3, K, prof, 2.0, cvs=0.01, chs=0.0)
    amp = 2 * np.mean(u[:, 1, 40] * np.cos(np.pi * sig)) / 0.01
    nu = 1e-6 + 0.01
    lam = (2 - 2 * math.cos(math.pi / K)) * K * K
    assert amp == pytest.approx(math.exp(-nu * lam * t), rel=2e-3)


def test_viscous_horizontal_mode_decays_at_the_diffusion_rate(oracle_mod):
    """Explicit horizontal viscous terms (diffusion, src/nhwave.F:6785-7141)
    with IHTURB = 1: a cross-channel profile U = U0 cos(pi y / W) decays by
    exp(-nu lambda t) more than the same run without viscosity (whose decay
    is the flux scheme's own), lambda = (2 - 2 cos(pi/N)) / dy^2."""
    N, K = 10, 4
    y = (np.arange(N) + 0.5) * 0.2
    prof = 0.01 * np.ones((K, 1)) * np.cos(np.pi * y / (N * 0.2))[None, :]
    amps = []
    for chs in (0.0, 0.05):
        t, u = _viscous_channel(oracle_mod, 40, N, K, prof, 1.5, cvs=0.0, chs=chs)
        amps.append(2 * np.mean(u[2, :, 20] * np.cos(np.pi * y / (N * 0.2))) / 0.01)
    lam = (2 - 2 * math.cos(math.pi / N)) / 0.04
    assert amps[1] / amps[0] == pytest.approx(math.exp(-0.05 * lam * t), rel=0.01)


def test_subgrid_eddy_viscosities_of_a_linear_flow(oracle_mod):
    """eval_turb with IVTURB = IHTURB = 2 (src/nhwave.F:6653-6665, 6686-6774)
    on U = a sigma + b x, V = W = 0 in a flat 1 m deep channel before the
    first sigma_transform (sigma slopes zero): dU/dsigma = a, so CmuVt =
    Cvs D dsig^2 |a| on the levels with both neighbours in the water; the
    only strain rate is dU/dx = b, so CmuHt = Chs dx dy |b| away from the
    side walls, mirrored into the ghosts.  The viscous time-step limit is
    VISCOUS_NUMBER min(dx^2, dy^2) over the largest CmuHt."""
    from nhwave_gb300 import default_params, fields as F
    M, N, K, dx, dy, a, b, cvs, chs = 16, 3, 6, 0.2, 0.25, 0.03, 0.002, 0.15, 0.12
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=dx, dy=dy, dt_ini=0.01, dt_max=1.0, tol=1e-10, itmax=2000,
                       viscous_flow=1, visc=1e-6, cvs=cvs, chs=chs, ivturb=2, ihturb=2)
    sig = (np.arange(K) + 0.5) / K
    x = (np.arange(M) + 0.5) * dx
    uvw = np.zeros((3, K, N, M))
    uvw[0] = a * sig[:, None, None] + b * x[None, None, :]
    o = oracle_mod.Oracle(p, np.ones(M * N), None, uvw.ravel())
    # the seeding viscosity Cmut_min = 0.09 Tke_min^2 / Eps_min (src/initialize.F:3178-3191)
    assert np.allclose(o.get(F.CMUVT), 9.0e-2 * 1e-9, rtol=1e-6)
    o.eval_turb(1)
    ng = F.NG
    cv, ch = o.get(F.CMUVT), o.get(F.CMUHT)
    # (sigma levels and dsig are default-real values of the reference: 1e-6)
    inner = (slice(ng + 1, ng + K - 1), slice(ng, ng + N), slice(ng, ng + M))
    assert cv[inner] == pytest.approx(np.full(cv[inner].shape, cvs / K ** 2 * a), rel=1e-6)
    cols = (slice(ng, ng + K), slice(ng, ng + N), slice(ng + 1, ng + M - 1))
    assert ch[cols] == pytest.approx(np.full(ch[cols].shape, chs * dx * dy * b), rel=1e-9)
    # ghosts mirror the interior across each side
    for gi in range(1, ng + 1):
        assert np.array_equal(ch[ng:ng + K, ng:ng + N, ng - gi], ch[ng:ng + K, ng:ng + N, ng + gi - 1])
        assert np.array_equal(ch[ng - gi, ng:ng + N, ng:ng + M], ch[ng + gi - 1, ng:ng + N, ng:ng + M])
        assert np.array_equal(ch[ng:ng + K, ng + N - 1 + gi, ng:ng + M], ch[ng:ng + K, ng + N - gi, ng:ng + M])
    assert o.estimate_dt() == 0
    top = np.abs(ch[ng:ng + K, ng:ng + N, ng:ng + M]).max()
    assert o.scalars().dt == pytest.approx(min(1.05 * 0.01, p.viscous_number * min(dx, dy) ** 2 / top), rel=1e-6)


def _ke_channel(oracle_mod, k0, e0, u_of_sigma=None, M=8, N=3, K=6, **kw):
    """Flat 1 m deep channel with the k-epsilon closure (IVTURB = IHTURB =
    10), uniform tke k0 and epsilon e0 in every cell, and an optional
    current U(sigma); returns the oracle."""
    from nhwave_gb300 import default_params, fields as F
    kw = dict(dict(visc=1e-6), **kw)
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=0.5, dy=0.5, dt_ini=0.01, dt_max=0.01, tol=1e-12, itmax=2000,
                       viscous_flow=1, ivturb=10, ihturb=10, **kw)
    uvw = np.zeros((3, K, N, M))
    if u_of_sigma is not None:
        uvw[0] = u_of_sigma((np.arange(K) + 0.5) / K)[:, None, None]
    o = oracle_mod.Oracle(p, np.ones(M * N), None, uvw.ravel())
    D = o.get(F.D)[None]
    shp = o.get(F.TKE).shape
    o.set(F.TKE, np.full(shp, k0)); o.set(F.EPS, np.full(shp, e0))
    o.set(F.DTKE, D * k0 * np.ones(shp)); o.set(F.DEPS, D * e0 * np.ones(shp))
    return o


def _ke_stage(o, istep=1):
    assert o.estimate_dt() == 0
    o.update_vars(); o.source_terms(); o.fluxes()
    assert o.eval_duvw(istep) == 0
    o.eval_turb(istep)


def test_ke_uniform_turbulence_decays_by_the_implicit_step(oracle_mod):
    """kepsilon_3D (src/nhwave.F:10030-11114) in still water with uniform
    tke k0 and epsilon e0: no production, advection or diffusion, so the
    first stage's implicit step gives eps1 = e0 / (1 + dt c2e e0 / k0) and
    k1 = k0 - dt eps1 above the bed level (whose wall function resets it),
    and CmuVt = cmiu k1^2 / eps1; CmuHt = CmuVt (IHTURB = 10)."""
    from nhwave_gb300 import fields as F
    k0, e0 = 1e-3, 1e-4
    o = _ke_channel(oracle_mod, k0, e0)
    _ke_stage(o)
    dt = o.scalars().dt
    ng, K = F.NG, 6
    c2e, cmiu = float(np.float32(1.92)), float(np.float32(0.09))
    e1 = e0 / (1 + dt * c2e * e0 / k0)
    k1 = k0 - dt * e1
    inner = (slice(ng + 1, ng + K), slice(ng, ng + 3), slice(ng, ng + 8))
    assert o.get(F.EPS)[inner] == pytest.approx(np.full((K - 1, 3, 8), e1), rel=1e-12)
    assert o.get(F.TKE)[inner] == pytest.approx(np.full((K - 1, 3, 8), k1), rel=1e-12)
    assert o.get(F.CMUVT)[inner] == pytest.approx(np.full((K - 1, 3, 8), cmiu * k1 * k1 / e1), rel=1e-12)
    assert np.array_equal(o.get(F.CMUHT), o.get(F.CMUVT))
    # still water over the bed: the wall function gives the floors there
    assert np.all(o.get(F.TKE)[ng, ng:ng + 3, ng:ng + 8] == pytest.approx(1e-9, rel=1e-6))


def test_ke_bed_wall_function_of_a_current(oracle_mod):
    """The bed condition of kepsilon_3D (src/nhwave.F:10776-10831): under a
    current, the first level's tke is u*^2 / sqrt(cmiu) and epsilon
    u*^3 / (Kappa Dz1), with u* = sqrt(Cdrag) |DU| / D and Cdrag the drag
    coefficient Cd0 capped by the viscous limit (Cmu + CmuVt) D / (Dz1 |DU|)."""
    from nhwave_gb300 import fields as F
    K = 6
    o = _ke_channel(oracle_mod, 1e-4, 1e-5, lambda s: 0.3 + 0.0 * s, K=K, visc=1e-3, bc_z0=5, ibot=1, cd0=0.003)
    cv_bed = o.get(F.CMUVT)[F.NG].copy()
    _ke_stage(o)
    ng = F.NG
    du = o.get(F.DU)[ng, ng + 1, ng + 3]
    D = o.get(F.D)[ng + 1, ng + 3]
    dz1 = 0.5 * D * float(np.float32(1.0) / np.float32(K))
    cd = min(0.003, (1e-3 + cv_bed[ng + 1, ng + 3]) / dz1 / (abs(du) + 1e-16) * D)
    us = math.sqrt(cd) * abs(du) / D
    kappa, cmiu = float(np.float32(0.41)), float(np.float32(0.09))
    assert o.get(F.TKE)[ng, ng + 1, ng + 3] == pytest.approx(us * us / math.sqrt(cmiu), rel=1e-12)
    assert o.get(F.EPS)[ng, ng + 1, ng + 3] == pytest.approx(us ** 3 / (kappa * dz1), rel=1e-12)


def test_ke_side_wall_function_along_a_friction_wall(oracle_mod):
    """The friction-wall condition of kepsilon_3D (BC_Y0 = 5, src/nhwave.F:
    10956-10987): along a south wall the first row takes tke u*^2 / sqrt(cmiu)
    and epsilon u*^3 / (kappa dy / 2) with u* = sqrt(Cd0) |(U, W)| of that
    row, on every level, mirrored into the ghost rows."""
    from nhwave_gb300 import fields as F
    K = 6
    o = _ke_channel(oracle_mod, 1e-4, 1e-5, lambda s: 0.2 + 0.0 * s, K=K, N=4, bc_y0=5, ibot=1, cd0=0.004)
    _ke_stage(o)
    ng = F.NG
    u, w = o.get(F.U)[:, ng, :], o.get(F.W)[:, ng, :]
    fric = math.sqrt(0.004) * np.sqrt(u * u + w * w)
    kap, cmiu = float(np.float32(0.41)), float(np.float32(0.09))
    cols, levs = slice(ng, ng + 8), slice(ng, ng + K)
    tk, ep = o.get(F.TKE), o.get(F.EPS)
    assert tk[levs, ng, cols] == pytest.approx((fric * fric / math.sqrt(cmiu))[levs, cols], rel=1e-12)
    assert ep[levs, ng, cols] == pytest.approx((fric ** 3 / (kap * 0.5 / 2.0))[levs, cols], rel=1e-12)
    assert np.array_equal(tk[levs, ng - 1, cols], tk[levs, ng, cols])


def test_ke_shear_produces_turbulence(oracle_mod):
    """The nonlinear production (src/nhwave.F:10139-10274): a sheared current
    U = 2 sigma keeps more tke above the bed level than still water from the
    same seeds, for every production form (PRODTYPE 1, 2, 3) and RNG."""
    from nhwave_gb300 import fields as F
    ng, K = F.NG, 6
    for prod, rng in ((3, 0), (2, 0), (1, 1)):
        kept = []
        for shear in (None, lambda s: 2.0 * s):
            o = _ke_channel(oracle_mod, 1e-4, 1e-5, shear, prod_type=prod, rng=rng)
            for _ in range(10):
                assert o.step() == 0
            kept.append(o.get(F.TKE)[ng + 1:ng + K, ng + 1, ng + 4].mean())
        assert kept[1] > 1.05 * kept[0], (prod, rng, kept)


def test_ke2_uniform_turbulence_decays_by_the_implicit_step(oracle_mod):
    """kepsilon (src/nhwave.F:11117-11524, IVTURB = 3) in still water with
    uniform tke k0 and epsilon e0: no production, advection or diffusion and,
    with no bed velocity, no wall function, so every level takes eps1 = e0 /
    (1 + dt c2e e0 / k0), k1 = k0 - dt eps1 and CmuVt = cmiu k1^2 / eps1."""
    from nhwave_gb300 import default_params, fields as F
    M, N, K, k0, e0 = 8, 3, 6, 1e-3, 1e-4
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=0.5, dy=0.5, dt_ini=0.01, dt_max=0.01, tol=1e-12, itmax=2000,
                       viscous_flow=1, visc=1e-6, ivturb=3, ihturb=10)
    o = oracle_mod.Oracle(p, np.ones(M * N))
    D = o.get(F.D)[None]
    shp = o.get(F.TKE).shape
    o.set(F.TKE, np.full(shp, k0)); o.set(F.EPS, np.full(shp, e0))
    o.set(F.DTKE, D * k0 * np.ones(shp)); o.set(F.DEPS, D * e0 * np.ones(shp))
    _ke_stage(o)
    dt = o.scalars().dt
    ng = F.NG
    e1 = e0 / (1 + dt * float(np.float32(1.92)) * e0 / k0)
    k1 = k0 - dt * e1
    inner = (slice(ng, ng + K), slice(ng, ng + N), slice(ng, ng + M))
    assert o.get(F.EPS)[inner] == pytest.approx(np.full((K, N, M), e1), rel=1e-12)
    assert o.get(F.TKE)[inner] == pytest.approx(np.full((K, N, M), k1), rel=1e-12)
    cmiu = float(np.float32(0.09))
    assert o.get(F.CMUVT)[inner] == pytest.approx(np.full((K, N, M), cmiu * k1 * k1 / e1), rel=1e-12)
    assert np.array_equal(o.get(F.CMUHT), o.get(F.CMUVT))


def test_les_smagorinsky_viscosity_and_smooth_wall_law(oracle_mod):
    """les_3D (src/nhwave.F:8545-8729) on a shear U = a sigma in a flat 1 m
    deep channel before the first sigma_transform: the only strain rate is
    S13 = a / (2 D), so CmuVt = (Cvs Delta)^2 a / D with Delta = (dx dy
    dsig D)^(1/3) on the levels whose neighbours are in the water, away
    from the end walls.  At the
    bed the smooth-wall law U/u* = ln(9 z u*/nu) / kappa at z = dsig D / 2
    gives CmuVt = kappa z u* (1 - exp(-z u*/(19 nu)))^2."""
    from scipy.optimize import brentq
    from nhwave_gb300 import default_params, fields as F
    M, N, K, dx, dy, a, cvs, nu = 12, 3, 6, 0.2, 0.25, 0.2, 0.1, 1e-6
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=dx, dy=dy, dt_ini=0.01, dt_max=1.0, tol=1e-10, itmax=2000,
                       viscous_flow=1, visc=nu, cvs=cvs, ivturb=20, ihturb=20, zob=1e-4)
    sig = (np.arange(K) + 0.5) / K
    uvw = np.zeros((3, K, N, M))
    uvw[0] = a * sig[:, None, None]
    o = oracle_mod.Oracle(p, np.ones(M * N), None, uvw.ravel())
    o.eval_turb(1)
    ng = F.NG
    cv = o.get(F.CMUVT)
    ds = float(np.float32(1.0) / np.float32(K))
    delta = (dx * dy * ds * 1.0) ** float(np.float32(1.0) / np.float32(3.0))
    # away from the end walls, whose mirrored U adds dU/dx
    inner = (slice(ng + 1, ng + K - 1), slice(ng, ng + N), slice(ng + 1, ng + M - 1))
    assert cv[inner] == pytest.approx(np.full(cv[inner].shape, (cvs * delta) ** 2 * a), rel=1e-6)
    kap, z, ub = float(np.float32(0.41)), 0.5 * ds, a * 0.5 / K
    x = brentq(lambda x: x * (math.log(9.0 * ub * z / nu) + math.log(x)) - kap, 1e-3, 1.0, xtol=1e-15)
    us = x * ub
    expect = kap * z * us * (1.0 - math.exp(-z * us / nu / 19.0)) ** 2
    assert cv[ng, ng:ng + N, ng:ng + M] == pytest.approx(np.full((N, M), expect), rel=1e-6)
    cols = (slice(ng, ng + N), slice(ng, ng + M))
    assert np.array_equal(cv[ng - 1][cols], cv[ng][cols]) and np.array_equal(o.get(F.CMUHT), cv)


def test_les_dyn_coefficient_of_a_linear_strain(oracle_mod):
    """les_dyn (src/nhwave.F:7989-8542) on U = a x in a flat 1 m deep channel
    before the first sigma_transform: S11 = a is the only strain rate, the
    test filter keeps linear fields, and the [1 2 1]/4 filter of u^2 adds
    (a dx)^2 / 2, so L11 = (a dx)^2 / 2 and M11 = 3 |S| a with |S| = sqrt(2)
    |a|.  The coefficient -L11 M11 / (2 M11^2) / Delta^2 is clipped to zero
    under stretching (a > 0); under compression (a < 0) it is dx^2 / (12
    sqrt(2) Delta^2) and CmuVt = C Delta^2 |S| = |a| dx^2 / 12 (times 27 x
    the default-real 1/27 of the smoothing filter), away from the walls,
    the bed and the surface."""
    from nhwave_gb300 import default_params, fields as F
    M, N, K, dx, dy = 32, 15, 8, 0.1, 0.5
    ng = F.NG
    out = []
    for a in (0.3, -0.3):
        p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=dx, dy=dy, dt_ini=0.01, dt_max=1.0, tol=1e-10,
                           itmax=2000, viscous_flow=1, visc=1e-6, ivturb=30, ihturb=30)
        x = (np.arange(M) + 0.5) * dx
        uvw = np.zeros((3, K, N, M))
        uvw[0] = a * (x - x.mean())[None, None, :]
        o = oracle_mod.Oracle(p, np.ones(M * N), None, uvw.ravel())
        o.eval_turb(1)
        out.append(o.get(F.CMUVT)[ng + 3:ng + K - 3, ng + N // 2, ng + 4:ng + M - 4])
    assert np.all(out[0] == 0.0)
    expect = 0.3 * dx * dx / 12.0 * 27.0 * float(np.float32(1.0) / np.float32(27.0))
    assert out[1] == pytest.approx(np.full(out[1].shape, expect), rel=1e-12)


def test_viscous_without_viscosity_is_the_inviscid_run(oracle_mod):
    """VISCOUS_FLOW = T with zero viscosities: the tridiagonal systems are the
    identity and the explicit terms vanish, so the run equals the inviscid
    one up to the seeding viscosity of the first stage (9e-11 m^2/s)."""
    from nhwave_gb300 import fields as F, scenarios as S
    outs = []
    for vf in (0, 1):
        p, d, e, u = S.make("tiny_c2")
        p.tol, p.itmax = 1e-12, 5000
        p.viscous_flow, p.visc, p.cvs, p.chs = vf, 0.0, 0.0, 0.0
        o = oracle_mod.Oracle(p, d, e, u)
        for _ in range(5):
            assert o.step() == 0
        outs.append(o.get(F.ETA)[o.shape.interior(F.ETA)])
    assert rel_l2(outs[1], outs[0]) < 1e-9


def test_bed_stress_slows_the_near_bed_flow(oracle_mod):
    """BC_Z0 = 2 (no slip) and 5 (friction law, src/nhwave.F:4806-4903 and
    the first rows of the implicit vertical step): the shear mode
    U = U0 cos(pi sigma), whose bed value is +U0, loses more of its amplitude
    over a no-slip or frictional bed than over a free-slip one."""
    K = 10
    sig = (np.arange(K) + 0.5) / K
    prof = 0.05 * np.cos(np.pi * sig)[:, None] * np.ones((1, 3))
    amps = {}
    for key, kw in (("free", dict(bc_z0=1)), ("noslip", dict(bc_z0=2)),
                    ("fric", dict(bc_z0=5, ibot=1, cd0=0.05))):
        t, u = _viscous_channel(oracle_mod, 40, 3, K, prof, 1.0, cvs=0.01, chs=0.0, **kw)
        amps[key] = 2 * np.mean(u[:, 1, 20] * np.cos(np.pi * sig)) / 0.05
        assert np.isfinite(u).all()
    assert amps["noslip"] < amps["free"] - 0.01
    assert amps["fric"] < amps["free"] - 0.002


def test_wave_current_inflow_carries_the_current(oracle_mod):
    """WAV_CUR (src/waves.F:706-756): the linear boundary wave of LEF_LIN on a
    current Cur_Wave ramped up as tanh(t/TRamp).  Until the current reaches
    the far side, the domain gains, over the plain LEF_LIN run, the volume
    the current carries in: Cur_Wave TRamp ln cosh(t/TRamp) h W."""
    from nhwave_gb300 import params as P, scenarios as S
    gain = []
    for wm in (P.WM_WAV_CUR, P.WM_LEF_LIN):
        p, d, e, u = S.make("tiny_flume_cur")
        p.wavemaker = wm
        p.tol, p.itmax = 1e-8, 5000
        o = oracle_mod.Oracle(p, d, e, u)
        m0 = o.mass()
        while o.scalars().time < 3.0:
            assert o.step() == 0
        gain.append(o.mass() - m0)
        t = o.scalars().time
    width = p.Nglob * p.dy
    expect = p.cur_wave * p.tramp * math.log(math.cosh(t / p.tramp)) * p.dep_wave * width
    assert gain[0] - gain[1] == pytest.approx(expect, rel=0.05)


def test_wall_friction_slows_the_flow_along_the_walls(oracle_mod):
    """BC_Y0 = BC_Yn = 5 (src/nhwave.F:4676-4691, 4737-4752): the ghosts
    along a wall take (1 - Phi) times the mirrored tangential velocity, Phi
    growing with the drag, so a flow along the channel loses more at the
    walls than between free-slip walls (Phi = 0)."""
    N, K = 10, 4
    y = (np.arange(N) + 0.5) * 0.2
    prof = 0.01 * np.ones((K, 1)) * np.cos(np.pi * y / (N * 0.2))[None, :]
    edge = {}
    for bc in (1, 5):
        t, u = _viscous_channel(oracle_mod, 40, N, K, prof, 1.0, cvs=0.0, chs=0.05, bc_y0=bc, bc_yn=bc,
                                ibot=1, cd0=5.0)
        edge[bc] = abs(u[2, 0, 20])
    assert edge[5] < 0.97 * edge[1]


def test_focused_group_boundary_elevation(oracle_mod):
    """FOCUSED (src/waves.F:638-692, components src/initialize.F:742-781):
    the boundary elevation is the sum of NWAVE linear components
    a_n cos(-k_n x_b - 2 pi f_n (t - t_b)), frequencies evenly spread over
    normalized_delta_f f_center, k_n from linear dispersion, a_n =
    Slope_group / NWAVE / k_n; recomputed here independently."""
    from nhwave_gb300 import scenarios as S
    p, d, e, u = S.make("tiny_flume_foc")
    p.tol, p.itmax = 1e-8, 5000
    o = oracle_mod.Oracle(p, d, e, u)
    pi = float(np.float32(3.141592653))
    g = float(np.float32(9.81))
    nw, h = p.nwave, p.depth_comp
    f = p.f_center - 0.5 * p.normalized_delta_f * p.f_center + np.arange(nw) * p.normalized_delta_f * p.f_center / (nw - 1)
    k = np.empty(nw)
    for n in range(nw):   # linear dispersion, to full precision
        sig2 = (2 * pi * f[n]) ** 2
        kk = 2 * pi / (math.sqrt(g * h) / f[n])
        for _ in range(60):
            kk -= (g * kk * math.tanh(kk * h) - sig2) / (g * kk * h * (1 - math.tanh(kk * h) ** 2) + g * math.tanh(kk * h))
        k[n] = kk
    a = p.slope_group / nw / k
    for _ in range(30):
        assert o.step() == 0
        t = o.scalars().time
        expect = np.sum(a * np.cos(-k * p.x_breaking - 2 * pi * f * (t - p.t_breaking)))
        assert _west_boundary_eta(o) == pytest.approx(expect, abs=1e-8)


def test_tide_sets_the_first_column_depth(oracle_mod):
    """LEF_TID (src/nhwave.F:5715-5750 with wl_bc :5145-5148): the boundary
    elevation is 0.5 A cos(2 pi t / 43200 - pi/2), and wl_bc sets D to
    Din = Hfx + Ein in the ghosts and the first interior column alike."""
    from nhwave_gb300 import fields as F, scenarios as S
    p, d, e, u = S.make("tiny_flume_tid")
    p.tol, p.itmax = 1e-8, 5000
    o = oracle_mod.Oracle(p, d, e, u)
    pi = float(np.float32(3.141592653))
    for _ in range(10):
        assert o.step() == 0
    t = o.scalars().time
    ein = 0.5 * p.amp_wave * math.cos(2.0 * pi / 43200.0 * t - pi / 2.0)
    D = o.get(F.D)
    assert np.allclose(D[2:-2, 0:3], p.dep_wave + ein, rtol=0, atol=1e-14)


def _pi_sp():
    return float(np.float32(3.141592653))


def test_east_linear_wave_sets_the_east_face_fluxes(oracle_mod):
    """RIG_LIN through BC_Xn = 3 (linear_wave_right_boundary, src/waves.F:762-803;
    flux_bc src/nhwave.F:2411-2416): the east face carries Din_Xn Uin_Xn with
    Ein_Xn = 0.5 A cos(pi/2 - sigma t), Din_Xn = Ein_Xn + h and the linear
    wave's velocity profile less its Stokes drift, level by level."""
    from nhwave_gb300 import fields as F, scenarios as S
    p, d, e, u = S.make("tiny_flume_rig")
    p.tol, p.itmax = 1e-10, 5000
    o = oracle_mod.Oracle(p, d, e, u)
    pi, g = _pi_sp(), float(np.float32(9.81))
    sigma = 2.0 * pi / p.per_wave
    k = oracle_mod.lib().orc_wave_number(o._h, sigma)
    h, A = p.dep_wave, p.amp_wave
    sd = g * A * A / ((2.0 * pi / k) / p.per_wave) / h / 8.0
    sigc = o.grid(6)
    f = p.Mglob + 2                      # the east face Iend1, 0-based
    for _ in range(30):
        assert o.step() == 0
        t = o.scalars().time
        E = 0.5 * A * math.cos(pi / 2 - sigma * t)
        Dn = E + h
        ex = o.get(F.EX)
        for kk in range(2, p.Kglob + 2):
            un = 0.5 * A * sigma * math.cosh(k * sigc[kk] * Dn) / math.sinh(k * h) * math.cos(pi / 2 - sigma * t) - sd
            assert ex[kk, 2:p.Nglob + 2, f] == pytest.approx(Dn * un, rel=1e-12, abs=1e-15)


def test_flux_lr_west_inflow_is_the_ramped_log_profile(oracle_mod):
    """FLUX_LR (flux_left_right_boundary, src/nhwave.F:5566-5712): the west
    face carries D Uin with eta = 0 and Uin = Ufric/kappa log(30 z/Zob)
    tanh(t/TRamp), Ufric = 0.115 kappa / log(30 D/Zob); the east side stays
    open (the volume in the domain grows by less than the volume let in)."""
    from nhwave_gb300 import fields as F, scenarios as S
    p, d, e, u = S.make("tiny_flux_lr")
    p.tol, p.itmax = 1e-10, 5000
    o = oracle_mod.Oracle(p, d, e, u)
    kappa, uavg = float(np.float32(0.41)), float(np.float32(0.115))
    sigc, dsig = o.grid(6), o.grid(5)
    D = float(o.get(F.HFX)[2, 2])         # Hfx(Ibeg, Jbeg): the inflow depth at eta = 0
    ufric = uavg * kappa / math.log(30.0 * D / p.zob)
    m0, inflow, t_prev = o.mass(), 0.0, 0.0
    for _ in range(40):
        assert o.step() == 0
        t = o.scalars().time
        ex = o.get(F.EX)
        flux = 0.0
        for kk in range(2, p.Kglob + 2):
            uin = ufric / kappa * math.log(30.0 * sigc[kk] * D / p.zob) * math.tanh(t / p.tramp)
            assert ex[kk, 2:p.Nglob + 2, 2] == pytest.approx(D * uin, rel=1e-12)
            flux += dsig[kk] * D * p.dy * uin * p.Nglob
        inflow += flux * (t - t_prev)
        t_prev = t
    gained = o.mass() - m0
    assert 0.0 < gained < inflow


@pytest.mark.parametrize("name", ["tiny_flume_jon", "tiny_flume_tma"])
def test_jonswap_boundary_elevation_has_the_spectrum_variance(name, oracle_mod):
    """LEF_JON / LEF_TMA (src/initialize.F:880-941, src/waves.F:566-623): the
    spectrum is scaled to m0 = Hm0^2/16, and each component's amplitude is
    Wh/2 with Wh = 2 sqrt(2 S df), so the boundary elevation's variance over a
    long record is sum S df = Hm0^2/16 (the components' frequencies are
    distinct, so their cross terms average out)."""
    from nhwave_gb300 import scenarios as S
    p, d, e, u = S.make(name)
    o = oracle_mod.Oracle(p, d, e, u)
    rec = []
    for n in range(6000):                   # 600 s at 0.1 s
        o.set_time(0.1 * n, 0.1, n)
        o.update_wave_bc()
        rec.append(o.inflow_eta()[3])
    rec = np.array(rec)
    assert abs(rec.mean()) < 0.02 * rec.std()
    assert rec.var() == pytest.approx(p.hm0 ** 2 / 16.0, rel=0.03)
    # the phases follow the seed: another seed gives another record with the same variance
    q = p.copy()
    q.wave_seed = p.wave_seed + 1
    o2 = oracle_mod.Oracle(q, d, e, u)
    o2.set_time(12.3, 0.1, 1)
    o2.update_wave_bc()
    o.set_time(12.3, 0.1, 1)
    o.update_wave_bc()
    assert o2.inflow_eta()[3] != o.inflow_eta()[3]


def test_spectral_inflow_follows_the_component_sum(oracle_mod):
    """LEF_SPC (random_wave_left_boundary, src/waves.F:376-513): the boundary
    elevation of row j is tanh(t/20) sum 0.5 Wh cos(pi/2 - 2 pi f t + yc_j
    sin(theta) k + phase), Wh = 2 sqrt(2 S df dtheta) with the centred band
    widths, k from the dispersion relation -- restated here in numpy."""
    from nhwave_gb300 import scenarios as S
    p, d, e, u = S.make("tiny_flume_spc")
    o = oracle_mod.Oracle(p, d, e, u)
    freq, dire, spc = S.spc_spectrum()
    ph = np.random.default_rng(9).uniform(0.0, 2.0 * np.pi, spc.size)
    o.set_wave_spectrum(freq, dire, spc, ph)
    pi = _pi_sp()

    def widths(a):
        w = np.empty_like(a)
        w[0], w[-1] = a[1] - a[0], a[-1] - a[-2]
        w[1:-1] = 0.5 * (a[2:] - a[:-2])
        return np.abs(w)
    nd = dire.size
    kw = np.array([oracle_mod.lib().orc_wave_number(o._h, 2.0 * pi / (1.0 / f)) for f in freq])
    wh = 2.0 * np.sqrt(2.0 * spc.reshape(freq.size, nd) * np.outer(widths(freq), widths(dire)))
    th = dire * pi / 180.0
    yc = o.grid(3)
    for t in (3.0, 17.5, 41.25):
        o.set_time(t, 0.1, 1)
        o.update_wave_bc()
        got = o.inflow_eta()
        for j in (2, 5, 9):
            lag = yc[j] * np.sin(th)[None, :] * kw[:, None] + ph.reshape(freq.size, nd)
            want = math.tanh(t / 20.0) * float(
                (0.5 * wh * np.cos(pi / 2 - (2.0 * pi * freq)[:, None] * t + lag)).sum())
            assert got[j] == pytest.approx(want, rel=1e-11, abs=1e-14)


def _snap(angle, k, width, irr):
    """The internal makers' direction search (src/source_terms.F:94-136,
    203-247), restated: the nearest direction whose cross-channel wave number
    n 2 pi / width the channel repeats."""
    pi, small = _pi_sp(), float(np.float32(1.0e-16))

    def search(sign):
        tmp3, nk = 0.0, 0
        while (tmp3 < angle) if sign > 0 else (tmp3 > angle):
            nk += 1
            tmp2 = nk * 2.0 * pi / width
            tmp3 = sign * (0.5 * pi - small) if tmp2 >= k else sign * math.asin(tmp2 / k)
        arg = (nk - 1) * 2.0 * pi / width / k
        tmp4 = math.asin(arg) if abs(arg) <= 1.0 else float("nan")
        return tmp4 if abs(tmp4 - angle) < abs(angle - tmp3) else tmp3
    if angle > 0.0:
        return search(1)
    if angle < 0.0 or not irr:
        return search(-1)
    return 0.0


@pytest.mark.parametrize("kind", ["spc", "irr"])
def test_internal_spectral_source_is_the_component_sum(kind, oracle_mod):
    """INT_SPC / INT_IRR (src/source_terms.F:71-302): in every cell of the
    source strip, SourceC = sum over components of C A / Source_Area cos(pi/2
    - sigma t + (dy/2 + yc_j) k sin(theta) + phase), theta the direction
    snapped to one the 4 m channel repeats, C = sigma / k, A = 2 sqrt(2 S
    ddir df) (INT_SPC) or 2 a (INT_IRR, whose first frequency takes the form
    2 C / Source_Area (A/2 cos + eta_mean), eta_mean = 0); restated here in
    numpy, and zero outside the strip."""
    from nhwave_gb300 import fields as F, scenarios as S
    p, d, e, u = S.make(f"tiny_int_{kind}")
    o = oracle_mod.Oracle(p, d, e, u)
    if kind == "spc":
        freq, dire, spc = S.spc_spectrum(8, 5, spread_deg=30.0)
        ph = np.random.default_rng(3).uniform(0.0, 2.0 * np.pi, spc.size)
    else:
        freq, dire, spc, ph = S.irr_components()
    o.set_wave_spectrum(freq, dire, spc, ph)
    pi = _pi_sp()

    def widths(a):
        w = np.empty_like(a)
        w[0], w[-1] = a[1] - a[0], a[-1] - a[-2]
        w[1:-1] = 0.5 * (a[2:] - a[:-2])
        return np.abs(w)
    nf, nd = freq.size, dire.size
    sig = 2.0 * pi / (1.0 / freq)
    kw = np.array([oracle_mod.lib().orc_wave_number(o._h, s) for s in sig])
    cel = (2.0 * pi / kw) / (1.0 / freq)
    if kind == "spc":
        amp = 2.0 * np.sqrt(2.0 * spc.reshape(nf, nd) * np.outer(widths(freq), widths(dire)))
    else:
        amp = 2.0 * spc.reshape(nf, nd)
    width = p.Nglob * p.dy
    th = np.array([[_snap(dd * pi / 180.0, kk, width, kind == "irr") for dd in dire] for kk in kw])
    # some directions snap to a non-zero cross-channel wave number that the channel repeats
    ky = kw[:, None] * np.sin(th)
    assert np.any(np.abs(ky) > 1.0)
    nz = np.abs(ky) > 1e-12
    assert np.allclose((ky[nz] / (2.0 * pi / width)), np.round(ky[nz] / (2.0 * pi / width)), atol=1e-9)
    xc, yc = o.grid(1), o.grid(3)
    D = o.get(F.D)
    strip = [i for i in range(2, 2 + p.Mglob) if p.xsource_west <= xc[i] <= p.xsource_east]
    assert strip
    area = sum(p.dx * D[3, i] for i in strip)   # Source_Area: row Jbeg + 1
    for t in (0.7, 4.25):
        o.set_time(t, 0.01, 1)
        o.source_terms()
        got = o.get(F.SOURCEC)
        for j in (2, 9, 17):
            arg = pi / 2 - sig[:, None] * t + (p.dy / 2.0 + yc[j]) * ky + ph.reshape(nf, nd)
            want = float((cel[:, None] * amp / area * np.cos(arg)).sum())
            for i in strip:
                assert got[j, i] == pytest.approx(want, rel=1e-10, abs=1e-12)
        assert np.all(got[2:-2, [i for i in range(2, 2 + p.Mglob) if i not in strip]] == 0.0)


@pytest.mark.parametrize("kind", ["jon", "tma"])
def test_internal_jonswap_source_is_the_component_sum(kind, oracle_mod):
    """INT_JON / INT_TMA (src/source_terms.F:305-340): SourceC = sum over the
    NumFreq components of C A / Source_Area cos(pi/2 - sigma t + phase),
    A = 2 sqrt(2 S DFreq), S the JONSWAP (TMA) spectrum at the band centres
    scaled to Hm0^2/16 -- restated here in numpy, with the phases given."""
    from nhwave_gb300 import fields as F, scenarios as S
    p, d, e, u = S.make(f"tiny_int_{kind}")
    o = oracle_mod.Oracle(p, d, e, u)
    nf = p.numfreq
    ph = np.random.default_rng(4).uniform(0.0, 2.0 * np.pi, nf)
    o.set_wave_phases(ph)
    pi, g = _pi_sp(), float(np.float32(9.81))
    df = (p.freq_max - p.freq_min) / nf
    f = p.freq_min + 0.5 * df + np.arange(nf) * df
    fp = 1.0 / p.tp
    s2 = np.where(f < fp, float(np.float32(0.07)) ** 2, float(np.float32(0.09)) ** 2)
    spec = g * g / f ** 5 * np.exp(-1.25 * (fp / f) ** 4) * float(np.float32(3.3)) ** np.exp(
        -0.5 * (f / fp - 1.0) ** 2 / s2)
    sig = 2.0 * pi / (1.0 / f)
    kw = np.array([oracle_mod.lib().orc_wave_number(o._h, s) for s in sig])
    if kind == "tma":
        h = p.dep_wave
        spec = spec * np.tanh(kw * h) ** 2 / (1.0 + 2 * kw * h / np.sinh(2.0 * kw * h))
    spec *= p.hm0 ** 2 / 16.0 / (spec * df).sum()
    dfreq = (p.freq_max - p.freq_min) / float(np.float32(nf))   # DFreq = (Freq_Max - Freq_Min) / float(NumFreq)
    amp = 2.0 * np.sqrt(2.0 * spec * dfreq)
    cel = (2.0 * pi / kw) / (1.0 / f)
    xc = o.grid(1)
    D = o.get(F.D)
    strip = [i for i in range(2, 2 + p.Mglob) if p.xsource_west <= xc[i] <= p.xsource_east]
    area = sum(p.dx * D[3, i] for i in strip)
    for t in (1.3, 9.7):
        o.set_time(t, 0.01, 1)
        o.source_terms()
        got = o.get(F.SOURCEC)
        want = float((cel * amp / area * np.cos(pi / 2 - sig * t + ph)).sum())
        for j in (2, 11):
            for i in strip:
                assert got[j, i] == pytest.approx(want, rel=1e-9, abs=1e-12)


def test_internal_cnoidal_source_has_zero_mean_over_a_period(oracle_mod):
    """INT_CON (src/source_terms.F:343-395): SourceC = 2 C / Source_Area
    (Ytrough + H cn^2(...)), and Ytrough puts the cnoidal profile's mean at
    zero, so over one period the source adds no volume: its mean over 400
    samples of a period is below 1e-3 of its peak; and its peak-to-trough
    range is 2 C H / Source_Area."""
    from nhwave_gb300 import fields as F, scenarios as S
    p, d, e, u = S.make("tiny_int_con")
    o = oracle_mod.Oracle(p, d, e, u)
    xc = o.grid(1)
    i = next(i for i in range(2, 2 + p.Mglob) if p.xsource_west <= xc[i] <= p.xsource_east)
    vals = []
    for n in range(400):
        o.set_time(p.per_wave * n / 400.0, 0.01, 1)
        o.source_terms()
        vals.append(o.get(F.SOURCEC)[5, i])
    vals = np.array(vals)
    assert abs(vals.mean()) < 1e-3 * np.abs(vals).max()
    D = o.get(F.D)
    strip = [q for q in range(2, 2 + p.Mglob) if p.xsource_west <= xc[q] <= p.xsource_east]
    area = sum(p.dx * D[3, q] for q in strip)
    # the cnoidal celerity lies between the shallow-water speeds of the trough and crest depths
    c_est = (vals.max() - vals.min()) * area / (2.0 * p.amp_wave)
    g = float(np.float32(9.81))
    assert math.sqrt(g * (p.dep_wave - p.amp_wave)) < c_est < math.sqrt(g * (p.dep_wave + p.amp_wave))
