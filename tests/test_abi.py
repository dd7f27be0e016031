"""The C-ABI library: loads, exports every declared symbol, validates
arguments on the host (no GPU needed for any of this)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    syms = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            syms |= set(re.findall(r"^\s*(?:int|const char \*|void)\s*\*?\s*(bh_\w+)\s*\(", txt, re.M))
    return syms


@pytest.fixture(scope="module")
def lib():
    from conftest import ensure_library

    return ensure_library().load_library()


def test_every_declared_symbol_exported(lib):
    from barneshut.gb300 import native

    syms = declared_symbols()
    assert len(syms) >= 20
    for s in sorted(syms):
        assert hasattr(lib, s), f"{s} declared in include/ but not exported"
    assert syms <= set(native.EXPORTS)


def test_grid_dim_matches_reference_formula(lib):
    from barneshut.implementations.base import reference_grid_dim

    for n in (2, 33, 600, 1000, 10_000, 1 << 20, 10_000_000):
        for ppb in (1, 2, 4, 23, 60, 1000):
            assert lib.bh_grid_dim(n, ppb) == reference_grid_dim(n, ppb), (n, ppb)
    assert lib.bh_grid_dim(10_000, 60) == 16
    assert lib.bh_grid_dim(10_000_000, 1000) == 120  # python-bh/data/frontera runs: 120 x 120


def _create(lib, n, G, **kw):
    from barneshut.gb300 import native

    prm = native.make_params(**kw)
    h = ctypes.c_void_p()
    na = (ctypes.c_longlong * len(n))(*n)
    ga = (ctypes.c_int * len(G))(*G)
    rc = lib.bh_plan_create(ctypes.byref(h), len(n), na, ga, ctypes.byref(prm))
    return rc, h


def test_plan_create_validates_on_host(lib):
    from barneshut.gb300 import native

    rc, h = _create(lib, [100], [4], softening=-1.0)
    assert rc == native.BH_ERR_INVALID and not h.value
    assert b"softening" in lib.bh_last_error(None)
    rc, h = _create(lib, [100], [4], group_dim=3)
    assert rc == native.BH_ERR_INVALID
    rc, h = _create(lib, [-5], [4])
    assert rc == native.BH_ERR_INVALID
    rc, h = _create(lib, [100], [40000])
    assert rc == native.BH_ERR_INVALID
    rc, h = _create(lib, [100], [4], precision=7)
    assert rc == native.BH_ERR_INVALID


def test_workspace_size_and_unbound_calls(lib):
    from barneshut.gb300 import native

    rc, h = _create(lib, [1000, 50], [8, 2], theta=0.5, softening=1e-3, cutoff_r2=0.0)
    assert rc == 0
    sz = ctypes.c_size_t()
    assert lib.bh_workspace_size(h, ctypes.byref(sz)) == 0
    # two FP64 state buffers dominate: >= 2 * 5 * 8 bytes per particle
    assert sz.value >= 1050 * 80
    # phases before bh_bind fail cleanly with a workspace error (no CUDA call)
    assert lib.bh_create_tree(h, None) == native.BH_ERR_WORKSPACE
    assert b"bh_bind" in lib.bh_last_error(h)
    assert lib.bh_step(h, 1, None) == native.BH_ERR_WORKSPACE
    # too-small workspace is refused before any device access
    assert lib.bh_bind(h, ctypes.c_void_p(256), 16, None) == native.BH_ERR_WORKSPACE
    assert lib.bh_plan_destroy(h) == 0


def test_missing_library_fails_loudly(monkeypatch):
    from barneshut.gb300 import native

    monkeypatch.setattr(native, "_lib", None)
    with pytest.raises(native.NativeLibraryError):
        native.load_library("/nonexistent/libbh_gb300.so")


def test_launch_count_host_logic(lib):
    """bh_kernels_per_step is host-only: a list-streaming plan builds no walk work items unless
    it carries the learned correction; a walking plan builds them (3 kernels: count, scan,
    fill).  No step graph exists before the first capture."""
    from barneshut.gb300 import native

    def count(**kw):
        rc, h = _create(lib, [100000], [64], theta=0.5, softening=1e-3, cutoff_r2=0.0, **kw)
        assert rc == 0
        c = ctypes.c_int()
        assert lib.bh_kernels_per_step(h, ctypes.byref(c)) == 0
        g = ctypes.c_int()
        assert lib.bh_graph_kernel_nodes(h, ctypes.byref(g)) == native.BH_ERR_INVALID
        assert lib.bh_plan_destroy(h) == 0
        return c.value

    stream = count()
    # prologue, bbox, place, box scan, 4 scatter kernels, stream items, summarize, lists, item
    # order (2), force
    assert stream == 14
    # walk items and the walk's own tick in, stream items and lists out
    assert count(flags=native.BH_FLAG_WALK) == stream + 3 + 1 - 4
    assert count(flags=native.BH_FLAG_LEARNED) == stream + 3


def _workspace(lib, n, G, **kw):
    rc, h = _create(lib, [n], [G], theta=0.5, softening=1e-4, cutoff_r2=0.0, **kw)
    assert rc == 0
    sz = ctypes.c_size_t()
    assert lib.bh_workspace_size(h, ctypes.byref(sz)) == 0
    assert lib.bh_plan_destroy(h) == 0
    return sz.value


def test_workspace_budget(lib):
    """Workspace of the list-streaming plans: the far-list slots dominate at small target groups
    (one 16-byte slot per cell a level's frontier can hold, 4 (TG/2 + 2/theta + 2)^2 at most,
    per level and group).  Budgets: N = 4,194,304 on 512 x 512 boxes, theta = 0.5 -- 1.26 GB with
    4 x 4 groups (the benchmark's tile), 6.1 GB with single-box groups; N = 16,777,216 on
    16384 x 16384 boxes needs 364 GB with 8 x 8 groups, more than one GPU holds; such grids take
    the pyramid walk (BH_FLAG_WALK), which keeps no lists: 38 GB, mostly the 358M pyramid cells'
    moments and records (80 B each)."""
    from barneshut.gb300 import native

    n4m = 1 << 22
    assert _workspace(lib, n4m, 512, group_dim=4) <= 1.26e9
    assert _workspace(lib, n4m, 512, group_dim=1) <= 6.1e9
    sizes = [_workspace(lib, n4m, 512, group_dim=t) for t in (1, 2, 4, 8)]
    assert sizes == sorted(sizes, reverse=True)
    big = _workspace(lib, 1 << 24, 16384, group_dim=8)
    assert 3.0e11 < big <= 3.7e11
    walk = _workspace(lib, 1 << 24, 16384, group_dim=8, flags=native.BH_FLAG_WALK)
    assert walk <= 3.9e10


def test_ctypes_binding_params_layout():
    """The standalone ctypes binding (implementations/gb300_ctypes.py) declares bh_params
    field for field like the package's own binding: same size, same offsets."""
    pytest.importorskip("torch")
    from barneshut.gb300 import native
    from barneshut.implementations import gb300_ctypes

    a, b = gb300_ctypes.BhParams, native.make_params().__class__
    assert ctypes.sizeof(a) == ctypes.sizeof(b)
    assert [f[0] for f in a._fields_] == [f[0] for f in b._fields_]
    for name, _ in a._fields_:
        assert getattr(a, name).offset == getattr(b, name).offset, name
