"""Regenerates the golden fixtures of tests/golden/ from the float64 oracle.

    python tests/golden/make_golden.py

Each case stores its seeded float32 inputs and the float64 oracle outputs
(oracle/nt_oracle.py, which restates the reference's rules) so that the GPU
tests compare against frozen vectors as well as against the live oracle.
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import nt_oracle as o  # noqa: E402


def fcn(m):
    return [m.Dense(512, W_std=1.5, b_std=0.05), m.Relu(), m.Dense(512, W_std=1.5, b_std=0.05),
            m.Relu(), m.Dense(1, W_std=1.5, b_std=0.05)]


def myrtle5(m):
    conv = lambda: m.Conv(1, (3, 3), padding='SAME', W_std=math.sqrt(2.), b_std=0.)
    return [conv(), m.Relu(), conv(), m.Relu(), m.AvgPool((2, 2), (2, 2)), conv(), m.Relu(),
            m.AvgPool((2, 2), (2, 2)), conv(), m.Relu()] + [m.AvgPool((2, 2), (2, 2))] * 3 + \
        [m.Flatten(), m.Dense(10, math.sqrt(2.), 0.)]


def conv_erf(m):
    return [m.Conv(3, (3, 3), padding='SAME', W_std=1.3, b_std=0.2), m.Erf(0.8, 1.1, 0.1),
            m.AvgPool((2, 2), (2, 2)), m.Conv(3, (2, 2), padding='VALID', W_std=1.2, b_std=0.1),
            m.Relu(), m.GlobalAvgPool(), m.Dense(1, 1.1, 0.05)]


CASES = {
    'fcn': (fcn, lambda r: r.standard_normal((24, 784)), 20, ('nngp', 'ntk', 'cov1', 'cov2')),
    'myrtle5': (myrtle5, lambda r: r.standard_normal((3, 32, 32, 3)), 2,
                ('nngp', 'ntk', 'cov1', 'cov2')),
    'conv_erf': (conv_erf, lambda r: r.standard_normal((4, 8, 8, 3)), 3,
                 ('nngp', 'ntk', 'cov1', 'cov2')),
}


def main():
    for name, (layers, gen, n1, get) in CASES.items():
        rng = np.random.default_rng(2024)
        x = gen(rng).astype(np.float32)
        x1, x2 = x[:n1], x[n1:]
        out = o.serial(*layers(o))(x1, x2, get)
        np.savez_compressed(os.path.join(HERE, f'{name}.npz'), x1=x1, x2=x2,
                            **{g: v for g, v in zip(get, out)})
        print(name, [np.asarray(v).shape for v in out])


if __name__ == '__main__':
    main()
