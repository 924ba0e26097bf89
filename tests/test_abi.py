"""C ABI: the library loads and exports every declared symbol; host-side
logic (generators, status strings, argument checks) works without a GPU."""
from __future__ import annotations

import hashlib
import json
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


def declared_symbols() -> set[str]:
    names = set()
    for h in ("gas_gb300.h", "gas_gb300_core.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"GAS_API\s+[\w\s\*]+?\b(gas_\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(gas_lib):
    names = declared_symbols()
    assert len(names) >= 35
    missing = [n for n in sorted(names) if not hasattr(gas_lib, n)]
    assert not missing, missing
    from vertexapi2_gb300 import _lib
    assert names == set(_lib.SIGNATURES), names ^ set(_lib.SIGNATURES)


def test_status_strings(gas_lib):
    assert gas_lib.gas_status_string(0) == b"ok"
    assert gas_lib.gas_status_string(4) == b"device wait timed out"


def test_engine_create_rejects_bad_program(gas_lib):
    import ctypes as C
    h = C.c_void_p()
    st = gas_lib.gas_engine_create(99, 0, None, C.byref(h))
    assert st != 0 and not h.value


def test_engine_calls_reject_null(gas_lib):
    assert gas_lib.gas_engine_run(None, 0, None) == 1
    assert gas_lib.gas_engine_get_results(None) == 1
    assert gas_lib.gas_core_set_active(None, 0, 1) == 1


def edge_hash(s, d, w=None):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(s, dtype="<i4").tobytes())
    h.update(np.ascontiguousarray(d, dtype="<i4").tobytes())
    if w is not None:
        h.update(np.ascontiguousarray(w, dtype="<i4").tobytes())
    return h.hexdigest()


def test_generators_reproduce_golden_inputs(gas_lib):
    from vertexapi2_gb300 import graphs
    idx = json.load(open(os.path.join(GOLDEN, "index.json")))["graphs"]
    gens = {
        "rmat8_sym": lambda: graphs.rmat(8, 16, seed=11, symmetrize=True, weights=(1, 255)),
        "rmat10_dir": lambda: graphs.rmat(10, 16, seed=12, weights=(1, 100)),
        "grid16": lambda: graphs.grid(16, 16, 0.15, seed=13),
        "grid40x30": lambda: graphs.grid(40, 30, 0.15, seed=14),
    }
    for name, gen in gens.items():
        g = gen()
        assert edge_hash(g.srcs, g.dsts, g.weights) == idx[name]["edge_sha256"], name


@pytest.mark.parametrize("sym", [False, True])
def test_rmat_properties(gas_lib, sym):
    from vertexapi2_gb300 import graphs
    g = graphs.rmat(12, 16, seed=5, symmetrize=sym, weights=(1, 255))
    s, d, w = g.srcs.astype(np.int64), g.dsts.astype(np.int64), g.weights
    assert g.n_vertices == 4096 and g.n_edges <= 16 * 4096 * (2 if sym else 1)
    assert np.all(s != d)                       # self-loops removed
    key = s * g.n_vertices + d
    assert np.all(np.diff(key) > 0)             # sorted by (src, dst), no duplicates
    assert w.min() >= 1 and w.max() <= 255
    if sym:
        rev = np.sort(d * g.n_vertices + s)
        assert np.array_equal(rev, key)         # symmetric
        order = np.argsort(d * g.n_vertices + s)
        assert np.array_equal(w[order], w)      # same weight both ways
    # power-law skew: the top vertex has far more than the mean degree
    deg = np.bincount(g.srcs, minlength=g.n_vertices)
    assert deg.max() > 20 * deg.mean()


def test_grid_properties(gas_lib):
    from vertexapi2_gb300 import graphs
    g = graphs.grid(64, 48, 0.15, seed=3)
    s, d = g.srcs.astype(np.int64), g.dsts.astype(np.int64)
    key = s * g.n_vertices + d
    assert np.all(np.diff(key) > 0)
    assert np.array_equal(np.sort(d * g.n_vertices + s), key)
    assert np.bincount(g.srcs, minlength=g.n_vertices).max() <= 4
    assert 0.5 * 64 * 48 < g.n_vertices <= 64 * 48
    # a single connected component
    import oracle
    lab, _ = oracle.port().cc(g.n_vertices, g.srcs, g.dsts)
    assert np.all(lab == 0)


def test_generator_argument_errors(gas_lib):
    from vertexapi2_gb300 import graphs
    from vertexapi2_gb300._lib import GasError
    with pytest.raises(GasError):
        graphs.rmat(0)
    with pytest.raises(GasError):
        graphs.grid(4, 4, p_delete=1.5)


def test_engine_without_device_reports_no_device(gas_lib):
    import ctypes as C
    if gas_lib.gas_device_supported(0):
        pytest.skip("a device is present")
    h = C.c_void_p()
    assert gas_lib.gas_engine_create(1, 0, None, C.byref(h)) == 7
    b = C.c_void_p()
    assert gas_lib.gas_batch_create(0, None, C.byref(b)) != 0


def test_server_argument_and_device_errors(gas_lib):
    """Configuration is checked before the device; without a device the
    server reports GAS_ERR_NO_DEVICE and hands out nothing."""
    import ctypes as C
    from vertexapi2_gb300._lib import ServerConfig
    h = C.c_void_p()
    assert gas_lib.gas_server_create(0, C.byref(ServerConfig(0, 256, 0)), C.byref(h)) == 1
    assert gas_lib.gas_server_create(0, C.byref(ServerConfig(4, 257, 0)), C.byref(h)) == 1
    assert gas_lib.gas_server_create(0, C.byref(ServerConfig(4, 256, -1)), C.byref(h)) == 1
    assert gas_lib.gas_server_create(0, None, None) == 1
    assert gas_lib.gas_server_destroy(None) == 0
    assert gas_lib.gas_server_submit(None, 0, 1, 0, None) == 1
    if not gas_lib.gas_device_supported(0):
        assert gas_lib.gas_server_create(0, None, C.byref(h)) == 7
        assert not h.value
