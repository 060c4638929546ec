"""The C-ABI library on a machine without a GPU: it loads, exports every entry
point declared in include/*.h, agrees with the ctypes struct images, and
rejects out-of-scope parameters on the host before touching the device."""
import ctypes
import glob
import os
import re

import pytest

from conftest import REPO


def _declared():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"\b(nhw_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_symbol(gpu_lib):
    declared = _declared()
    assert len(declared) >= 20
    missing = [n for n in declared if not hasattr(gpu_lib, n)]
    assert not missing, missing
    from nhwave_gb300 import lib
    assert sorted(lib.EXPORTS) == declared


def test_abi_sizes_match_ctypes(gpu_lib):
    from nhwave_gb300.params import NhwParams, NhwScalars
    a, b = ctypes.c_int32(), ctypes.c_int32()
    assert gpu_lib.nhw_abi_sizes(ctypes.byref(a), ctypes.byref(b)) == 0
    assert a.value == ctypes.sizeof(NhwParams)
    assert b.value == ctypes.sizeof(NhwScalars)


def test_status_strings(gpu_lib):
    from nhwave_gb300 import lib
    assert lib.status_string(0) == "ok"
    assert "DT_MIN" in lib.status_string(lib.ERR_DT_MIN)


@pytest.mark.parametrize("field,value", [("bc_x0", 3), ("bc_xn", 3), ("bc_yn", 6), ("bc_z0", 3), ("Kglob", 65),
                                         ("wavemaker", -1)])
def test_out_of_scope_options_rejected_on_host(field, value, gpu_lib):
    from nhwave_gb300 import default_params, lib
    p = default_params(**{field: value})
    h = ctypes.c_void_p()
    st = gpu_lib.nhw_create(ctypes.byref(p), ctypes.byref(h))
    assert st == lib.ERR_UNSUPPORTED and not h.value


@pytest.mark.parametrize("fields", [dict(ivturb=4), dict(ivturb=31, ihturb=10), dict(ivturb=11),
                                    dict(ivturb=2, ihturb=0), dict(ivturb=10, ihturb=3)])
def test_viscous_closures_outside_the_path_rejected(fields, gpu_lib):
    """VISCOUS_FLOW = T runs with IVTURB 1 (constant viscosity), 2 (subgrid
    model), 3 / 10 (2-D / 3-D k-epsilon) or 20 / 30 (Smagorinsky / dynamic
    LES) and IHTURB 1, 2 or >= 10; other codes are rejected on the host."""
    from nhwave_gb300 import default_params, lib
    p = default_params(viscous_flow=1, **fields)
    h = ctypes.c_void_p()
    assert gpu_lib.nhw_create(ctypes.byref(p), ctypes.byref(h)) == lib.ERR_UNSUPPORTED and not h.value
    for bad in (dict(schmidt=0.0), dict(viscous_number=0.0)):
        p = default_params(viscous_flow=1, **bad)
        assert gpu_lib.nhw_create(ctypes.byref(p), ctypes.byref(h)) == lib.ERR_ARG and not h.value


@pytest.mark.parametrize("field,value", [("Mglob", 0), ("dx", 0.0), ("precision", 7), ("time_order", 4),
                                         ("krylov_kernel", 3)])
def test_bad_arguments_rejected(field, value, gpu_lib):
    from nhwave_gb300 import default_params, lib
    p = default_params(**{field: value})
    h = ctypes.c_void_p()
    assert gpu_lib.nhw_create(ctypes.byref(p), ctypes.byref(h)) == lib.ERR_ARG


def test_null_arguments(gpu_lib):
    from nhwave_gb300 import lib
    assert gpu_lib.nhw_create(None, None) == lib.ERR_ARG
    assert gpu_lib.nhw_step(None, None, None, None) == lib.ERR_ARG
    assert gpu_lib.nhw_destroy(None) == lib.ERR_ARG


@pytest.mark.parametrize("fields,status", [
    (dict(bc_x0=3, wavemaker=8, nwave=1, f_center=1.0, depth_comp=0.5), "ERR_ARG"),      # FOCUSED, one component
    (dict(bc_x0=3, wavemaker=8, nwave=4, f_center=0.0, depth_comp=0.5), "ERR_ARG"),      # no centre frequency
    (dict(bc_x0=3, wavemaker=6, amp_wave=0.0), "ERR_ARG"),                                # cnoidal of zero height
    (dict(bc_x0=3, wavemaker=6, amp_wave=0.02, per_wave=1.5, dep_wave=0.5), "ERR_ARG"),  # cnoidal in deep water
    (dict(bc_y0=5, ibot=3), "ERR_UNSUPPORTED"),                                           # unknown Ibot
    (dict(bc_z0=5, ibot=2, zob=0.0), "ERR_ARG"),                                          # roughness height 0
    (dict(bc_x0=3, wavemaker=1), "ERR_UNSUPPORTED"),                                      # inflow without a LEF_ maker
    (dict(bc_xn=3), "ERR_UNSUPPORTED"),                                                   # east inflow
])
def test_added_options_checked_on_host(fields, status, gpu_lib):
    """The boundary-wave, wall/bed and FOCUSED options are checked on the host
    before any device work: impossible values are NHW_ERR_ARG (the reference
    would stop or run with NaN), options outside the path NHW_ERR_UNSUPPORTED."""
    from nhwave_gb300 import default_params, lib
    p = default_params(**fields)
    h = ctypes.c_void_p()
    assert gpu_lib.nhw_create(ctypes.byref(p), ctypes.byref(h)) == getattr(lib, status) and not h.value


def test_reference_example_inputs_pass_the_host_checks(gpu_lib):
    """Every example input of the reference that the Python reader places
    inside the path also passes nhw_create's host checks: on a machine
    without a GPU the call gets as far as the device and fails there
    (NHW_ERR_CUDA), never with NHW_ERR_UNSUPPORTED or NHW_ERR_ARG.  The
    others are rejected as unsupported.  Reads the reference checkout that
    NHWAVE_REFERENCE names, if set."""
    import glob
    from nhwave_gb300 import lib, params as P
    root = os.environ.get("NHWAVE_REFERENCE")
    if not root:
        pytest.skip("NHWAVE_REFERENCE (a reference checkout) is not set")
    files = sorted(glob.glob(os.path.join(root, "**", "input*.txt"), recursive=True))
    if not files:
        pytest.skip("no input files under NHWAVE_REFERENCE")
    for f in files:
        p = P.read_input(f)
        h = ctypes.c_void_p()
        st = gpu_lib.nhw_create(ctypes.byref(p), ctypes.byref(h))
        if P.unsupported_reason(p) is None:
            assert st not in (lib.ERR_UNSUPPORTED, lib.ERR_ARG), (f, st)
            if st == 0:
                gpu_lib.nhw_destroy(h)
        else:
            assert st == lib.ERR_UNSUPPORTED, (f, st)
