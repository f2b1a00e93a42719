"""Autotuner bookkeeping on the host: network keys and the JSON cache."""
import importlib
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture()
def tune(tmp_path, monkeypatch):
    monkeypatch.setenv('NT_GB300_TUNE_CACHE', str(tmp_path / 'tune.json'))
    import nt_gb300.tune as t
    t = importlib.reload(t)
    yield t
    t.clear()


def test_network_key_is_stable_and_parameter_sensitive():
    from nt_gb300 import stax, tune
    a = stax.serial(stax.Conv(1, (3, 3), padding='SAME', W_std=1.5), stax.Relu(),
                    stax.Flatten(), stax.Dense(1))[2]
    b = stax.serial(stax.Conv(1, (3, 3), padding='SAME', W_std=1.5), stax.Relu(),
                    stax.Flatten(), stax.Dense(1))[2]
    c = stax.serial(stax.Conv(1, (3, 3), padding='SAME', W_std=1.4), stax.Relu(),
                    stax.Flatten(), stax.Dense(1))[2]
    assert tune.network_key(a) == tune.network_key(b)
    assert tune.network_key(a) != tune.network_key(c)


def test_cache_round_trip(tune, tmp_path):
    tune._store('k1', {'tile': 16})
    data = json.loads((tmp_path / 'tune.json').read_text())
    assert data == {'k1': {'tile': 16}}
    tune.clear()
    tune._loaded = False
    tune._load()
    assert tune._cache['k1'] == {'tile': 16}
