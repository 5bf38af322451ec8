"""The allocation-free neighbour entry point (sp_neighbors_noalloc).

Callers that cannot allocate device memory while they run (code recording a
CUDA stream capture, hosts with their own fixed device-memory arena) pass
their own device buffers; the call keeps its cell-list scratch in a static
device array.  This file is collected last so that a failure here stops a
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


@pytest.mark.parametrize("case", ["rdme3d", "dam"])
def test_noalloc_neighbors_equal_existing_entry_point(lib, case):
    torch = pytest.importorskip("torch")
    from spatialpy_gb300.engine import Engine
    if case == "rdme3d":
        sc = S.config_rdme_3d(n=14, nA=10, nB=10)
        kmax = 64
    else:
        sc = S.config_dam_break(spacing_div=16, num_steps=10).copy(static_domain=True)
        kmax = 64
    # the existing path: sp_create + sp_get_neighbors
    with Engine(sc) as eng:
        want = eng.neighbors(0, kmax)
    n = sc.num_particles
    cuda = torch.device("cuda", 0)
    dev = {
        "x": torch.tensor(sc.x, dtype=torch.float64, device=cuda),
        "mass": torch.tensor(sc.mass, dtype=torch.float64, device=cuda),
        "rho": torch.tensor(sc.rho, dtype=torch.float64, device=cuda),
        "count": torch.zeros(n, dtype=torch.int32, device=cuda),
        "idx": torch.full((n, kmax), -1, dtype=torch.int32, device=cuda),
        "dist": torch.zeros((n, kmax), dtype=torch.float64, device=cuda),
        "dw": torch.zeros((n, kmax), dtype=torch.float64, device=cuda),
        "dij": torch.zeros((n, kmax), dtype=torch.float64, device=cuda),
    }
    lo = sc.x.min(axis=0)
    hi = sc.x.max(axis=0)
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


def test_noalloc_rejects_sizes_beyond_its_limit(lib):
    err = C.create_string_buffer(256)
    one = (C.c_double * 3)(0, 0, 0)
    big = (C.c_double * 3)(1, 1, 1)
    dummy = C.c_void_p(16)
    rc = lib.sp_neighbors_noalloc(dummy, 262145, 3, 0.1, dummy, dummy, one, big, 32, dummy,
                                  dummy, None, None, None, None, err, len(err))
    assert rc == abi.SP_E_INVALID and b"262,144" in err.value
    rc = lib.sp_neighbors_noalloc(dummy, 1000, 3, 1e-3, dummy, dummy, one, big, 32, dummy,
                                  dummy, None, None, None, None, err, len(err))
    assert rc == abi.SP_E_INVALID and b"524,288" in err.value
