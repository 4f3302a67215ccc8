"""Host-side checks of the C ABI library that need no GPU: it loads, exports
every entry point include/gofr_gb300.h declares, computes exact bin
thresholds and the reference's exact thread fold, and fails cleanly without
a device."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "gofr_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gofr_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(built_engine):
    from analisi_gb300 import engine
    decl = declared_symbols()
    assert len(decl) >= 15
    for name in decl:
        assert hasattr(built_engine, name), name
    assert sorted(engine.EXPORTED) == decl


def test_every_entry_point_cites_what_it_replaces():
    """Each declaration's comment names the reference interface it replaces
    (path:line in the analisi tree) or says that there is no counterpart."""
    src = open(os.path.join(ROOT, "include", "gofr_gb300.h")).read()
    decls = re.finditer(r"/\*((?:(?!\*/).)*)\*/\s*(?:const\s+)?[a-z_ ]+\*?\s*(gofr_[a-z0-9_]+)\s*\(",
                        src, flags=re.S)
    seen = set()
    for m in decls:
        comment, name = m.group(1), m.group(2)
        seen.add(name)
        if name == "gofr_last_error":
            continue  # the message accessor of the C ABI's own error convention
        assert re.search(r"\.(cpp|h|py):\d+", comment) or "counterpart" in comment, name
    assert seen >= set(declared_symbols()) - {"gofr_last_error"}


def test_no_device_is_a_clean_error(built_engine):
    from conftest import HAS_GPU
    if HAS_GPU:
        pytest.skip("a GPU is present")
    ctx = ctypes.c_void_p()
    rc = built_engine.gofr_ctx_create(ctypes.byref(ctx), 0)
    assert rc != 0 and not ctx.value
    assert b"no context" in built_engine.gofr_last_error(None)


@pytest.mark.parametrize("rmin,rmax,nbin", [(0.0, 3.5, 200), (0.7, 3.5, 200), (0.0, 12.0, 400),
                                            (0.0, 15.0, 500), (0.0, 10.0, 250), (0.1, 1.0, 9),
                                            (0.0, 1.0, 10), (0.0, 3.8, 200)])
def test_thresholds_are_exact(built_engine, oracle_mod, rmin, rmax, nbin):
    """th[b] is the smallest d2 the reference bins into >= b (th[0]: smallest
    counted d2, th[nbin]: just above the largest)."""
    from analisi_gb300 import engine
    th = engine.bin_thresholds(rmin, rmax, nbin)
    for b in range(nbin + 1):
        x = th[b]
        below = np.nextafter(x, -np.inf)
        ob, pb = oracle_mod.bin_of(x, rmin, rmax, nbin), oracle_mod.bin_of(below, rmin, rmax, nbin)
        if b == 0:
            assert ob == 0 and pb == -1
        elif b == nbin:
            assert ob == -1 and pb == nbin - 1
        else:
            assert ob >= b and pb < b


def test_thresholds_negative_rmin(built_engine, oracle_mod):
    """rmin < 0: the rmin^2 filter starts the window at bin (|rmin|-rmin)/dr."""
    from analisi_gb300 import engine
    th = engine.bin_thresholds(-1.0, 2.0, 30)
    assert th[0] == 1.0
    assert oracle_mod.bin_of(th[0], -1.0, 2.0, 30) == 20
    assert oracle_mod.bin_of(np.nextafter(th[0], -np.inf), -1.0, 2.0, 30) == -1


def test_unsupported_bin_map(built_engine):
    from analisi_gb300 import engine
    with pytest.raises(engine.GofrError):
        engine.bin_thresholds(2.0, 1.0, 10)


@pytest.mark.parametrize("nts,skip", [(700, 10), (20, 3), (1800, 4), (37, 1), (5, 8), (100, 7)])
def test_exact_thread_fold(built_engine, oracle_mod, nts, skip):
    """gofr_counts_to_buffer rebuilds the reference's double buffer (incr added
    k times per thread, threads folded in order) in O(binades) per bin."""
    from analisi_gb300 import engine
    rng = np.random.default_rng(nts * 31 + skip)
    c = rng.integers(0, 5000, size=(4, 3, 5, 7)).astype(np.uint64)
    c[0, 0, 0, 0] = 0
    a = engine.counts_to_buffer(c, nts, skip, nparts=4)
    b = oracle_mod.fold_buffer(c, oracle_mod.incr(nts, skip))
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    t = engine.counts_to_buffer(c[0], nts, skip, nparts=0)
    assert np.array_equal(t, c[0].astype(np.float64) * oracle_mod.incr(nts, skip))
    one = engine.counts_to_buffer(c[:1], nts, skip, nparts=1)
    assert np.array_equal(one.view(np.uint64),
                          oracle_mod.fold_buffer(c[:1], oracle_mod.incr(nts, skip)).view(np.uint64))


def test_exact_fold_large_counts(built_engine):
    """Large k: the closed form must match plain repeated addition."""
    from analisi_gb300 import engine
    inc = 1.0 / 450
    for k in (1, 2, 3, 1000, 123457, 2_000_003):
        s = 0.0
        for _ in range(k):
            s += inc
        got = engine.counts_to_buffer(np.array([[k]], dtype=np.uint64), 1800, 4, nparts=0)
        assert got[0, 0] == k * inc
        one = engine.counts_to_buffer(np.array([[[k]]], dtype=np.uint64), 1800, 4, nparts=1)
        assert one[0, 0] == s, k
        got2 = engine.counts_to_buffer(np.array([[[k]], [[0]]], dtype=np.uint64), 1800, 4,
                                       nparts=2)
        assert got2[0, 0] == s, k
