"""Shared fixtures.  `gpu` tests call the CUDA library through its C ABI and compare
with the CPU oracle; everything else runs on the CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle.oracle import oracle
    return oracle()


@pytest.fixture(scope="session")
def ref_lib():
    from oracle.oracle import reference
    r = reference()
    if r is None:
        pytest.skip("reference harness not built on this machine")
    return r


@pytest.fixture(scope="session")
def gpu_lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from nbpg_gb300 import _lib, build_ext
    if not os.path.exists(_lib.LIB_PATH):
        build_ext.build()
    return _lib.lib()


_DATA = {}


def dataset(dtype: str, metric: str, n: int = 3000, dims: int = 32, nq: int = 150, R: int = 24, L: int = 32,
            seed: int = 0):
    """Seeded small dataset + graph built by the oracle (Vamana, 1 pass)."""
    key = (dtype, metric, n, dims, nq, R, L, seed)
    if key in _DATA:
        return _DATA[key]
    from nbpg_gb300 import synth
    from oracle.oracle import oracle
    if dtype == "u8":
        base, q = synth.u8_mixture(n, nq, dim=dims, n_centres=24, seed=seed)
    elif dtype == "i8":
        base, q = synth.i8_unit_mixture(n, nq, dim=dims, n_centres=24, seed=seed)
    else:
        b8, q8 = synth.u8_mixture(n, nq, dim=2 * dims, n_centres=24, seed=seed)
        base, q = synth.pack_u4(b8 >> 4), synth.pack_u4(q8 >> 4)
    g, _, _, _ = oracle().build_graph(dtype, metric, base, R=R, L=L, VL=max(L + 8, 40), num_split=0, num_passes=1,
                                      max_alpha=1.2)
    _DATA[key] = (base, q, g)
    return _DATA[key]
