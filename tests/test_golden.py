"""Golden fixtures: the oracle reproduces them (CPU); the GPU kernels match them (GPU)."""
import os

import numpy as np
import pytest

from oracle import nt_oracle as o

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
import importlib.util  # noqa: E402

_spec = importlib.util.spec_from_file_location('make_golden', os.path.join(HERE, 'make_golden.py'))
G = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(G)


@pytest.mark.parametrize('name', sorted(G.CASES))
def test_oracle_reproduces_fixture(name):
    layers, _, _, get = G.CASES[name]
    f = np.load(os.path.join(HERE, f'{name}.npz'))
    out = o.serial(*layers(o))(f['x1'], f['x2'], get)
    for g, v in zip(get, out):
        np.testing.assert_allclose(v, f[g], rtol=1e-12, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize('name', sorted(G.CASES))
def test_gpu_matches_fixture(nt, name):
    layers, _, _, get = G.CASES[name]
    f = np.load(os.path.join(HERE, f'{name}.npz'))
    out = nt.stax.serial(*layers(nt.stax))[2](f['x1'], f['x2'], get)
    for g, v in zip(get, out):
        got = v.detach().cpu().numpy()
        want = f[g]
        err = np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-30))
        assert err < 1e-5, (g, err)
