"""The allocation-free neighbour entry point (sp_neighbors_noalloc).

Some callers cannot call cudaMalloc while they run: hosts that hand out all
device memory from their own fixed arena, and loops that cannot take the
device-wide synchronisation of cudaMalloc/cudaFree.  They pass their own
device buffers; the call keeps its cell-list scratch in a static device
array shared by every call.  These tests compare it with sp_get_neighbors
(itself pinned to the oracle and to the reference's neighbour lists) on two
calls in a row.  This file is collected last so that a failure here stops a
run only after every other test has run; it also passes on its own in a
fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from spatialpy_gb300 import abi
from spatialpy_gb300 import scenario as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from spatialpy_gb300 import build
    build.build()
    return abi.load_library()


def _call(lib, sc, kmax, dev, lo, hi, err):
    return lib.sp_neighbors_noalloc(
        C.c_void_p(dev["x"].data_ptr()), sc.num_particles, sc.dimension, sc.h,
        C.c_void_p(dev["mass"].data_ptr()), C.c_void_p(dev["rho"].data_ptr()),
        (C.c_double * 3)(*lo), (C.c_double * 3)(*hi), kmax,
        C.c_void_p(dev["count"].data_ptr()), C.c_void_p(dev["idx"].data_ptr()),
        C.c_void_p(dev["dist"].data_ptr()), C.c_void_p(dev["dw"].data_ptr()),
        C.c_void_p(dev["dij"].data_ptr()), None, err, len(err))


def _device_buffers(torch, sc, kmax):
    n = sc.num_particles
    cuda = torch.device("cuda", 0)
    return {
        "x": torch.tensor(sc.x, dtype=torch.float64, device=cuda),
        "mass": torch.tensor(sc.mass, dtype=torch.float64, device=cuda),
        "rho": torch.tensor(sc.rho, dtype=torch.float64, device=cuda),
        "count": torch.zeros(n, dtype=torch.int32, device=cuda),
        "idx": torch.full((n, kmax), -1, dtype=torch.int32, device=cuda),
        "dist": torch.zeros((n, kmax), dtype=torch.float64, device=cuda),
        "dw": torch.zeros((n, kmax), dtype=torch.float64, device=cuda),
        "dij": torch.zeros((n, kmax), dtype=torch.float64, device=cuda),
    }


def _case(case):
    if case == "rdme3d":     # 3-D lattice, h = 2.2 s: interior particles have 32 neighbours
        return S.config_rdme_3d(n=14, nA=10, nB=10)
    return S.config_dam_break(spacing_div=16, num_steps=10).copy(static_domain=True)


@pytest.mark.parametrize("case,kmax,box", [("rdme3d", 32, "tight"), ("rdme3d", 128, "tight"),
                                           ("dam", 64, "tight"), ("dam", 32, "inside")])
def test_noalloc_neighbors_equal_existing_entry_point(lib, case, kmax, box):
    """Two calls in a row equal sp_get_neighbors exactly (kmax 32 and 64
    run one kernel width each, 128 the widest); with the box shrunk inside
    the point cloud the outside particles fall into edge cells and every
    list is still complete."""
    torch = pytest.importorskip("torch")
    from spatialpy_gb300.engine import Engine
    sc = _case(case)
    # the existing path: sp_create + sp_get_neighbors
    with Engine(sc) as eng:
        want = eng.neighbors(0, kmax)
    n = sc.num_particles
    dev = _device_buffers(torch, sc, kmax)
    lo = sc.x.min(axis=0)
    hi = sc.x.max(axis=0)
    if box == "inside":
        span = hi - lo
        lo, hi = lo + 0.3 * span, hi - 0.3 * span
    err = C.create_string_buffer(256)
    for call in range(2):                       # two calls in a row share the scratch
        for k in ("count", "dist", "dw", "dij"):
            dev[k].zero_()
        dev["idx"].fill_(-1)
        torch.cuda.synchronize()
        rc = _call(lib, sc, kmax, dev, lo, hi, err)
        assert rc == abi.SP_OK, err.value.decode()
        torch.cuda.synchronize()
        cnt = dev["count"].cpu().numpy()
        np.testing.assert_array_equal(cnt, want[0], err_msg=f"call {call}")
        got = [dev[k].cpu().numpy() for k in ("idx", "dist", "dw", "dij")]
        for i in range(n):
            c = cnt[i]
            for a, b in zip(got, want[1:]):
                np.testing.assert_array_equal(a[i, :c], b[i, :c], err_msg=f"call {call} p {i}")


def test_noalloc_reports_lists_longer_than_kmax_then_recovers(lib):
    """kmax below the largest neighbour count gives SP_E_UNSUPPORTED; the
    next call with a sufficient kmax starts from a cleared flag and is
    exact."""
    torch = pytest.importorskip("torch")
    from spatialpy_gb300.engine import Engine
    sc = _case("rdme3d")
    err = C.create_string_buffer(256)
    lo, hi = sc.x.min(axis=0), sc.x.max(axis=0)
    dev = _device_buffers(torch, sc, 8)
    rc = _call(lib, sc, 8, dev, lo, hi, err)
    assert rc == abi.SP_E_UNSUPPORTED and b"kmax" in err.value
    with Engine(sc) as eng:
        want = eng.neighbors(0, 64)
    dev = _device_buffers(torch, sc, 64)
    rc = _call(lib, sc, 64, dev, lo, hi, err)
    assert rc == abi.SP_OK, err.value.decode()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dev["count"].cpu().numpy(), want[0])
