"""GPU: nhw_estimate_dt_noalloc against nhw_estimate_dt.

nhw_estimate_dt_noalloc serves callers that cannot let the library allocate
device memory: a host model whose fields already live on the GPU in memory
owned by another runtime (OpenACC, CUDA Fortran, a framework's caching
allocator), for which the cudaMalloc/cudaFree of a handle would synchronise
the device and break a memory budget fixed up front.  It takes the caller's
device arrays and keeps its reduction scratch in a fixed device array of the
library.  These tests call it through the C interface, with arrays that the
test (the caller) allocates, and require the same dt, bit for bit, as the
handle-based estimate_dt on the same state -- on consecutive calls, which
share that scratch.  This file sorts last so that a run stopping at its first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dsig(K):
    # uniform sigma levels: 1.0/float(Kglob) in default real (src/initialize.F:1702), with ghosts
    return np.full(K + 4, np.float64(np.float32(1.0) / np.float32(K)))


def _noalloc_dt(L, torch, g, dt_old, out, device="cuda"):
    """Upload U, V, W, D and dsig as the caller's device arrays; one call."""
    from nhwave_gb300 import fields as F
    p = g.params
    arrs = [torch.from_numpy(np.ascontiguousarray(g.get(getattr(F, n)), dtype=np.float64)).to(device)
            for n in ("U", "V", "W", "D")]
    arrs.append(torch.from_numpy(_dsig(p.Kglob)).to(device))
    torch.cuda.synchronize()
    st = L.nhw_estimate_dt_noalloc(*[a.data_ptr() for a in arrs], p.Mglob, p.Nglob, p.Kglob,
                                   p.dx, p.dy, p.cfl, dt_old, p.dt_max, out.data_ptr(), None)
    torch.cuda.synchronize()
    return st, float(out.cpu()[0])


@pytest.mark.parametrize("name", ["tiny_c2", "c2"])
def test_noalloc_dt_matches_estimate_dt(name, gpu_lib):
    torch = pytest.importorskip("torch")
    from nhwave_gb300 import lib, scenarios as S
    p, d, e, u = S.make(name, precision=0, seed=5)
    p.tol, p.itmax = 1e-10, 5000
    assert p.ivgrd == 1
    g = lib.Scenario(p, d, e, u)
    L = lib.load()
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    for call in range(2):          # two calls in a row, on two different states
        g.step()
        dt_old = g.scalars().dt
        st, got = _noalloc_dt(L, torch, g, dt_old, out)
        assert st == lib.OK, lib.last_error()
        assert g.estimate_dt() == lib.OK
        want = g.scalars().dt
        assert got == want, f"call {call}: {got!r} != {want!r}"
        assert g.scalars().dt_old == dt_old
    g.close()


def test_noalloc_rejects_oversize_and_host_arrays(gpu_lib):
    torch = pytest.importorskip("torch")
    from nhwave_gb300 import lib
    L = lib.load()
    # every buffer holds the (4+4) x (4+4) x (2+4) ghosted arrays of the small calls
    buf = torch.zeros(1024, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    ptr = buf.data_ptr()
    # 4097 x 4096 x 1 interior cells: one column block past the 16,777,216-cell limit
    st = L.nhw_estimate_dt_noalloc(ptr, ptr, ptr, ptr, ptr, 4097, 4096, 1, 1.0, 1.0, 0.5, 1.0, 1.0,
                                   out.data_ptr(), None)
    assert st == lib.ERR_ARG
    assert "16777216" in lib.last_error()
    host = np.zeros(1024)
    st = L.nhw_estimate_dt_noalloc(host.ctypes.data, ptr, ptr, ptr, ptr, 4, 4, 2, 1.0, 1.0, 0.5, 1.0, 1.0,
                                   out.data_ptr(), None)
    assert st == lib.ERR_ARG
    st = L.nhw_estimate_dt_noalloc(None, ptr, ptr, ptr, ptr, 4, 4, 2, 1.0, 1.0, 0.5, 1.0, 1.0,
                                   out.data_ptr(), None)
    assert st == lib.ERR_ARG


def test_noalloc_skips_nan_like_estimate_dt(gpu_lib):
    """A NaN depth in one cell gives NaN candidates there; both entry points
    skip them, as the reference's `if (dzonw < tmp2) tmp2 = dzonw` does, and
    return the same dt from the other cells."""
    torch = pytest.importorskip("torch")
    from nhwave_gb300 import fields as F, lib, scenarios as S
    p, d, e, u = S.make("tiny_c1", precision=0, seed=5)
    g = lib.Scenario(p, d, e, u)
    L = lib.load()
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    assert g.step() == lib.OK
    for cell in [(3, 7), (4, 20)]:          # interior (j, i) of the ghosted 2-D array
        dt_old = g.scalars().dt
        D = g.get(F.D).copy()
        D[cell] = np.nan
        g.set(F.D, D)
        st, got = _noalloc_dt(L, torch, g, dt_old, out)
        assert st == lib.OK, lib.last_error()
        assert np.isfinite(got)
        assert g.estimate_dt() == lib.OK     # takes dt_old from the handle's dt
        assert got == g.scalars().dt
    g.close()


def test_noalloc_rejects_another_devices_arrays(gpu_lib):
    """Arrays on a GPU other than the current one are refused (their loads
    would fault without peer access); needs two visible GPUs."""
    torch = pytest.importorskip("torch")
    if torch.cuda.device_count() < 2:
        pytest.skip("one GPU visible")
    from nhwave_gb300 import lib
    L = lib.load()
    other = torch.zeros(1024, dtype=torch.float64, device="cuda:1")
    ptr = torch.zeros(1024, dtype=torch.float64, device="cuda:0").data_ptr()
    out = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    torch.cuda.set_device(0)
    st = L.nhw_estimate_dt_noalloc(other.data_ptr(), ptr, ptr, ptr, ptr, 4, 4, 2, 1.0, 1.0, 0.5, 1.0, 1.0,
                                   out.data_ptr(), None)
    assert st == lib.ERR_ARG
    assert "current device" in lib.last_error()
