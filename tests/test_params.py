"""input.txt reader (src/mod_util.F:8-463 / read_input src/initialize.F:141-1321)."""
import pytest

SAMPLE = """! INPUT FILE FOR NHWAVE
TITLE = test
Mglob = 1024
Nglob = 64
Kglob = 20
DX = 0.025
DY = 0.05
IVGRD = 1
GRD_R = 1.1
DT_INI = 0.01000
DT_MIN = 0.00001
DT_MAX = 60.0000
SIM_STEPS = 100000000
TOTAL_TIME = 20.0
CFL = 0.5
FROUDE_CAP = 100.0
NON_HYDRO = T
MinDep = 1.e-3
ISOLVER = 2
ITMAX = 1000
TOL = 1.e-8
BC_X0 = 1
BC_Xn = 1
BC_Y0 = 1
BC_Yn = 1
BC_Z0 = 1
WAVEMAKER = INT_LIN
AMP = 0.01
PER = 2.02
DEP = 0.4
THETA = 0.0
CUR = 0.0
Xsource_West = 4.0   ! a comment
Xsource_East = 4.2
Ysource_Suth = 0.0
Ysource_Nrth = 3.2
SPONGE_ON = T
Sponge_West_Width =  2.0
Sponge_East_Width =  2.0
Sponge_South_Width = 0.0
Sponge_North_Width = 0.0
TIME_ORDER = THIRD
HLLC = F
VISCOUS_FLOW = F
BAROTROPIC = T
"""


def test_read_input(tmp_path):
    from nhwave_gb300 import params as P
    f = tmp_path / "input.txt"
    f.write_text(SAMPLE)
    p = P.read_input(str(f))
    assert (p.Mglob, p.Nglob, p.Kglob) == (1024, 64, 20)
    assert p.dx == 0.025 and p.dy == 0.05 and p.min_dep == 1e-3 and p.tol == 1e-8
    assert p.wavemaker == P.WM_INT_LIN and p.per_wave == 2.02 and p.xsource_west == 4.0
    assert p.sponge_on == 1 and p.sponge_west_width == 2.0 and p.non_hydro == 1
    assert p.time_order == 3 and p.total_time == 20.0
    assert P.unsupported_reason(p) is None


def test_missing_key_halts(tmp_path):
    from nhwave_gb300 import params as P
    f = tmp_path / "input.txt"
    f.write_text(SAMPLE.replace("DX = 0.025\n", ""))
    with pytest.raises(ValueError, match="DX"):
        P.read_input(str(f))


def test_out_of_scope_reason(tmp_path):
    from nhwave_gb300 import params as P
    f = tmp_path / "input.txt"
    f.write_text(SAMPLE.replace("HLLC = F", "HLLC = T"))
    p = P.read_input(str(f))
    assert p.hllc == 1 and P.unsupported_reason(p) is None
    f.write_text(SAMPLE.replace("BC_Z0 = 1", "BC_Z0 = 3"))
    assert "BC_Z0" in P.unsupported_reason(P.read_input(str(f)))
    f.write_text(SAMPLE.replace("BC_Z0 = 1", "BC_Z0 = 5"))
    p = P.read_input(str(f))
    assert p.bc_z0 == 5 and P.unsupported_reason(p) is None
    # a generator name the reference does not know either is rejected, not run as NONE
    f.write_text(SAMPLE.replace("WAVEMAKER = INT_LIN", "WAVEMAKER = INT_XYZ"))
    p = P.read_input(str(f))
    assert p.wavemaker == P.WM_OTHER and "WAVEMAKER" in P.unsupported_reason(p)
    # every internal maker of the reference is on the path (src/source_terms.F)
    for name, wm in (("INT_CON", P.WM_INT_CON), ("INT_JON", P.WM_INT_JON), ("INT_TMA", P.WM_INT_TMA),
                     ("INT_SPC", P.WM_INT_SPC), ("INT_IRR", P.WM_INT_IRR)):
        f.write_text(SAMPLE.replace("WAVEMAKER = INT_LIN", "WAVEMAKER = " + name))
        p = P.read_input(str(f))
        assert p.wavemaker == wm and P.unsupported_reason(p) is None, name
    # the cnoidal, Stokes and JONSWAP boundary waves are on the path, through BC_X0 = 3
    for name, wm in (("LEF_CON", P.WM_LEF_CON), ("LEF_STK", P.WM_LEF_STK), ("LEF_JON", P.WM_LEF_JON)):
        f.write_text(SAMPLE.replace("WAVEMAKER = INT_LIN", "WAVEMAKER = " + name))
        p = P.read_input(str(f))
        assert p.wavemaker == wm
        p.bc_x0 = 3
        assert P.unsupported_reason(p) is None


def test_irr2d_reader(tmp_path):
    """irr2d.txt (src/initialize.F:835-876): counts, frequencies, directions,
    then amplitudes and phases, direction fastest."""
    import numpy as np
    from nhwave_gb300 import params as P
    f = tmp_path / "irr2d.txt"
    vals = [2, 3, 0.5, 0.8, -10.0, 0.0, 10.0] + [0.001 * q for q in range(6)] + [0.1 * q for q in range(6)]
    f.write_text("\n".join(str(v) for v in vals))
    freq, dire, amp, ph = P.read_irr2d(str(f))
    assert list(freq) == [0.5, 0.8] and list(dire) == [-10.0, 0.0, 10.0]
    assert np.allclose(amp, [0.001 * q for q in range(6)]) and np.allclose(ph, [0.1 * q for q in range(6)])
    f.write_text("\n".join(str(v) for v in vals[:-1]))
    with pytest.raises(ValueError):
        P.read_irr2d(str(f))


def test_reference_example_inputs_where_present():
    """The reference's own example input files, read by the host reader: all
    fall inside the GPU path (the viscous ones with the 3-D k-epsilon model)
    but those with the open south/north/east sides of BC = 4, which are
    rejected with their reason.  Reads the reference checkout that
    NHWAVE_REFERENCE names, if set."""
    import glob
    import os
    from nhwave_gb300 import params as P
    root = os.environ.get("NHWAVE_REFERENCE")
    if not root:
        pytest.skip("NHWAVE_REFERENCE (a reference checkout) is not set")
    files = sorted(glob.glob(os.path.join(root, "**", "input*.txt"), recursive=True))
    if not files:
        pytest.skip("no input files under NHWAVE_REFERENCE")
    inside = 0
    for f in files:
        p = P.read_input(f)
        reason = P.unsupported_reason(p)
        if 4 in (p.bc_x0, p.bc_xn, p.bc_y0, p.bc_yn):
            assert reason and "BC_" in reason, f
        else:
            assert reason is None, (f, reason)
            inside += 1
    assert inside >= 14


def test_reader_takes_the_added_keys(tmp_path):
    """The keys of the viscous, bed, wall and FOCUSED options reach nhw_params
    (src/initialize.F:357, 385-392, 466-468, 614, 709-719)."""
    from nhwave_gb300 import params as P
    f = tmp_path / "input.txt"
    extra = """
IVTURB = 1
IHTURB = 1
VISCOSITY = 2.e-6
Schmidt = 0.7
Cvs = 0.003
Chs = 0.02
RNG = T
VISCOUS_NUMBER = 0.2
Ibot = 2
Cd0 = 0.004
Zob = 2.e-4
"""
    text = (SAMPLE.replace("BC_Z0 = 1", "BC_Z0 = 5").replace("BC_Y0 = 1", "BC_Y0 = 5")
            .replace("VISCOUS_FLOW = F", "VISCOUS_FLOW = T") + extra)
    f.write_text(text)
    p = P.read_input(str(f))
    assert p.viscous_flow == 1 and p.ivturb == 1 and p.ihturb == 1 and p.rng == 1
    assert (p.visc, p.schmidt, p.cvs, p.chs, p.viscous_number) == (2e-6, 0.7, 0.003, 0.02, 0.2)
    assert (p.bc_z0, p.bc_y0, p.ibot, p.cd0, p.zob) == (5, 5, 2, 0.004, 2e-4)
    assert P.unsupported_reason(p) is None
    f.write_text(text.replace("IVTURB = 1", "IVTURB = 10").replace("IHTURB = 1", "IHTURB = 10") + "PRODTYPE = 2\n")
    q = P.read_input(str(f))
    assert (q.ivturb, q.ihturb, q.prod_type) == (10, 10, 2) and P.unsupported_reason(q) is None
    f.write_text(text.replace("IVTURB = 1", "IVTURB = 40"))
    assert "IVTURB" in P.unsupported_reason(P.read_input(str(f)))
    foc = SAMPLE.replace("WAVEMAKER = INT_LIN", "WAVEMAKER = FOCUSED") + """
nwave = 12
Component_Amp_Type = 1
k_center = 4.0
f_center = 1.1
x_breaking = 6.0
t_breaking = 9.0
Slope_group = 0.3
normalized_delta_f = 0.75
depth_comp = 0.6
"""
    f.write_text(foc)
    p = P.read_input(str(f))
    assert p.wavemaker == P.WM_FOCUSED and p.nwave == 12 and p.component_amp_type == 1
    assert (p.k_center, p.f_center, p.x_breaking, p.t_breaking) == (4.0, 1.1, 6.0, 9.0)
    assert (p.slope_group, p.normalized_delta_f, p.depth_comp) == (0.3, 0.75, 0.6)


def test_reader_takes_the_jonswap_keys(tmp_path):
    """Hm0, Tp, Freq_Min, Freq_Max and NumFreq reach nhw_params for LEF_JON /
    LEF_TMA (src/initialize.F:888-892); FLUX_LR and RIG_LIN are read as such."""
    from nhwave_gb300 import params as P
    f = tmp_path / "input.txt"
    f.write_text(SAMPLE.replace("WAVEMAKER = INT_LIN", "WAVEMAKER = LEF_TMA") +
                 "\nHm0 = 0.05\nTp = 2.0\nFreq_Min = 0.2\nFreq_Max = 1.5\nNumFreq = 60\n")
    p = P.read_input(str(f))
    assert p.wavemaker == P.WM_LEF_TMA
    assert (p.hm0, p.tp, p.freq_min, p.freq_max, p.numfreq) == (0.05, 2.0, 0.2, 1.5, 60)
    for name, wm in (("FLUX_LR", P.WM_FLUX_LR), ("RIG_LIN", P.WM_RIG_LIN)):
        f.write_text(SAMPLE.replace("WAVEMAKER = INT_LIN", "WAVEMAKER = " + name))
        assert P.read_input(str(f)).wavemaker == wm
