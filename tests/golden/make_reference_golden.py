"""Golden vectors from the reference itself: runs neural-tangents 0.6.6's own stax and predict
code on the JAX stand-in of oracle/jax_stand_in (JAX is not installable here; the stand-in
restates, in numpy, the JAX primitives that path calls) and writes its outputs next to the
oracle's fixtures.

    python tests/golden/make_reference_golden.py [path of the neural-tangents checkout]

Writes, in float64 (the reference under jax_enable_x64, inputs cast to float64):
  <name>_reference.npz   for every case of make_golden.CASES (the same float32 inputs as the
                         oracle's fixtures): x1, x2 and the reference's nngp / ntk / cov1 / cov2;
  reference_cases.npz    KERNEL_CASES below (activations, paddings, strides, pools, readouts,
                         x2 = None, full- and diagonal-spatial kernels), keys '<case>/<name>';
  reference_random.npz   nngp / ntk of the 40 seeded random networks of random_networks()
                         (their specs and inputs are regenerated from the seed) and the
                         diagonal_spatial requirement the reference derives for each
                         (input, output as Bool values), its init_fn's output shape for x1
                         and the ValueError text of a diagonal_spatial=True request ('' when
                         the network serves it), keys 'net<i>/<name>';
  reference_predictions.npz  gradient_descent_mse at t = None / inf / a scalar / an array of
                         times, gradient_descent_mse_ensemble and gp_inference (means and
                         covariances), keys '<case>/<name>', and the kernels they were
                         computed from ('kernels/dd_nngp', 'kernels/td_ntk', ...).
The case definitions are importable without the reference (tests/test_golden.py rebuilds each
network on the oracle and compares).
"""
import math
import os
import sys
import types
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DEFAULT_REFERENCE = '/root/reference'


def _fc(m, *acts):
    """Dense -> act -> Dense -> act ... -> Dense(1), W / b varied per layer."""
    out = []
    for i, a in enumerate(acts):
        out += [m.Dense(8, 1.3 - 0.1 * i, 0.1 + 0.05 * i), a(m)]
    return out + [m.Dense(1, 1.1, 0.05)]


KERNEL_CASES = {
    # name: (layers(m), x1 shape, x2 shape or None, get, kernel_fn kwargs)
    'fc_abrelu_leaky': (lambda m: _fc(m, lambda m: m.ABRelu(-0.3, 1.1),
                                      lambda m: m.LeakyRelu(0.2)),
                        (5, 7), (4, 7), ('nngp', 'ntk', 'cov1', 'cov2'), {}),
    'fc_abs_relu_stabilized': (lambda m: _fc(m, lambda m: m.Abs(),
                                             lambda m: m.Relu(do_stabilize=True)),
                               (5, 7), (4, 7), ('nngp', 'ntk', 'cov1', 'cov2'), {}),
    'fc_gelu_sin': (lambda m: _fc(m, lambda m: m.Gelu(), lambda m: m.Sin(1.3, 0.7, 0.2)),
                    (5, 7), (4, 7), ('nngp', 'ntk', 'cov1', 'cov2'), {}),
    'fc_cos_rbf': (lambda m: _fc(m, lambda m: m.Cos(0.9, 1.1, -0.3), lambda m: m.Rbf(0.6)),
                   (5, 7), (4, 7), ('nngp', 'ntk', 'cov1', 'cov2'), {}),
    'fc_erf_same_inputs': (lambda m: _fc(m, lambda m: m.Erf(0.7, 1.2, 0.1), lambda m: m.Relu()),
                           (6, 7), None, ('nngp', 'ntk', 'cov1'), {}),
    'conv_valid_strided_flatten': (
        lambda m: [m.Conv(1, (3, 2), strides=(2, 1), padding='VALID', W_std=1.3, b_std=0.1),
                   m.Relu(), m.Conv(1, (2, 2), padding='SAME', W_std=1.2, b_std=0.05),
                   m.Erf(), m.Flatten(), m.Dense(1, 1.1, 0.1)],
        (2, 7, 6, 2), (3, 7, 6, 2), ('nngp', 'ntk', 'cov1', 'cov2'), {}),
    'conv_circular_pools': (
        lambda m: [m.Conv(1, (3, 3), padding='CIRCULAR', W_std=1.4, b_std=0.1), m.Relu(),
                   m.AvgPool((2, 2), (1, 1), 'SAME', normalize_edges=False),
                   m.Conv(1, (3, 3), padding='SAME', W_std=1.2, b_std=0.2), m.Gelu(),
                   m.SumPool((2, 2), (2, 2)), m.GlobalSumPool(), m.Dense(1, 1.3, 0.1)],
        (2, 6, 6, 3), (3, 6, 6, 3), ('nngp', 'ntk', 'cov1', 'cov2'), {}),
    'conv_avgpool_normalized_gap': (
        lambda m: [m.Conv(1, (3, 3), padding='SAME', W_std=1.3, b_std=0.1), m.Relu(),
                   m.AvgPool((3, 3), (2, 2), 'SAME', normalize_edges=True),
                   m.Conv(1, (2, 2), padding='VALID', W_std=1.2, b_std=0.05), m.Sin(1.1, 0.9, 0.3),
                   m.GlobalAvgPool(), m.Dense(1, 1.2, 0.1)],
        (2, 7, 7, 2), (2, 7, 7, 2), ('nngp', 'ntk', 'cov1', 'cov2'), {}),
    'cnn_full_spatial_kernel': (
        lambda m: [m.Conv(1, (3, 3), padding='SAME', W_std=1.3, b_std=0.1), m.Relu(),
                   m.Conv(1, (2, 3), padding='VALID', W_std=1.1, b_std=0.2), m.Erf()],
        (2, 5, 6, 3), (3, 5, 6, 3), ('nngp', 'ntk', 'cov1', 'cov2'),
        {'diagonal_spatial': False}),
    'cnn_diagonal_spatial_kernel': (
        lambda m: [m.Conv(1, (3, 3), padding='SAME', W_std=1.3, b_std=0.1), m.Relu(),
                   m.Conv(1, (2, 3), padding='VALID', W_std=1.1, b_std=0.2), m.Rbf(0.4)],
        (2, 5, 6, 3), (3, 5, 6, 3), ('nngp', 'ntk', 'cov1', 'cov2'),
        {'diagonal_spatial': True}),
    'myrtle_like_16_same_inputs': (
        lambda m: [m.Conv(1, (3, 3), padding='SAME', W_std=math.sqrt(2.), b_std=0.), m.Relu(),
                   m.Conv(1, (3, 3), padding='SAME', W_std=math.sqrt(2.), b_std=0.), m.Relu(),
                   m.AvgPool((2, 2), (2, 2)),
                   m.Conv(1, (3, 3), padding='SAME', W_std=math.sqrt(2.), b_std=0.), m.Relu(),
                   m.AvgPool((2, 2), (2, 2)), m.Flatten(), m.Dense(10, math.sqrt(2.), 0.)],
        (3, 16, 16, 3), None, ('nngp', 'ntk', 'cov1'), {}),
    'myrtle10_32': (lambda m: _myrtle10(m), (2, 32, 32, 3), (1, 32, 32, 3),
                    ('nngp', 'ntk', 'cov1', 'cov2'), {}),
    'myrtle5_32_same_inputs': (lambda m: _myrtle5(m), (3, 32, 32, 3), None,
                               ('nngp', 'ntk', 'cov1'), {}),
    'conv1d_pool_gap': (
        lambda m: [m.Conv(1, (3,), padding='SAME', W_std=1.3, b_std=0.1), m.Relu(),
                   m.AvgPool((2,), (2,)), m.Conv(1, (2,), padding='VALID', W_std=1.2, b_std=0.05),
                   m.Erf(), m.GlobalAvgPool(), m.Dense(1, 1.1, 0.1)],
        (2, 9, 3), (3, 9, 3), ('nngp', 'ntk', 'cov1', 'cov2'), {}),
    'conv1d_circular_strided_same_inputs': (
        lambda m: [m.Conv(1, (3,), strides=(2,), padding='CIRCULAR', W_std=1.3, b_std=0.1),
                   m.Gelu(), m.Flatten(), m.Dense(1, 1.1, 0.1)],
        (3, 9, 3), None, ('nngp', 'ntk', 'cov1'), {}),
    'fc_standard_parameterization': (
        lambda m: [m.Dense(8, W_std=1.3, b_std=0.1, parameterization='standard', s=(2, 3)),
                   m.Relu(), m.Dense(8, W_std=1.2, b_std=0.2, parameterization='standard'),
                   m.Erf(), m.Dense(1, W_std=1.1, b_std=0.05, parameterization='standard', s=(3, 1))],
        (5, 7), (4, 7), ('nngp', 'ntk', 'cov1', 'cov2'), {}),
    'conv_standard_parameterization': (
        lambda m: [m.Conv(1, (3, 3), padding='SAME', W_std=1.3, b_std=0.1,
                          parameterization='standard', s=(1, 2)), m.Relu(),
                   m.Conv(1, (2, 2), padding='VALID', W_std=1.2, b_std=0.05,
                          parameterization='standard', s=(2, 1)), m.Relu(),
                   m.GlobalAvgPool(), m.Dense(1, 1.1, 0.05, parameterization='standard')],
        (2, 6, 6, 3), (3, 6, 6, 3), ('nngp', 'ntk', 'cov1', 'cov2'), {}),
}


def _myrtle5(m):
    """Myrtle-5 as benchmarked: Conv3x3 + Relu x2, AvgPool, Conv + Relu, AvgPool, Conv + Relu,
    AvgPool x3, Flatten, Dense (W_std = sqrt 2, b_std = 0)."""
    conv = lambda: m.Conv(1, (3, 3), padding='SAME', W_std=math.sqrt(2.), b_std=0.)
    pool = lambda: m.AvgPool((2, 2), (2, 2))
    return [conv(), m.Relu(), conv(), m.Relu(), pool(), conv(), m.Relu(), pool(), conv(),
            m.Relu(), pool(), pool(), pool(), m.Flatten(), m.Dense(10, math.sqrt(2.), 0.)]


def _myrtle10(m):
    """Myrtle-10: Conv3x3 + Relu blocks [3, 3, 3] with AvgPool(2, 2) between them,
    GlobalAvgPool, Dense (W_std = sqrt 2, b_std = 0)."""
    conv = lambda: m.Conv(1, (3, 3), padding='SAME', W_std=math.sqrt(2.), b_std=0.)
    layers = []
    for i in range(3):
        for _ in range(3):
            layers += [conv(), m.Relu()]
        if i < 2:
            layers.append(m.AvgPool((2, 2), (2, 2)))
    return layers + [m.GlobalAvgPool(), m.Dense(10, math.sqrt(2.), 0.)]


def kernel_inputs(name):
    _, s1, s2, _, _ = KERNEL_CASES[name]
    rng = np.random.default_rng(zlib.crc32(name.encode()))  # stable across processes
    x1 = rng.standard_normal(s1)
    x2 = None if s2 is None else rng.standard_normal(s2)
    return x1, x2


_ACTS = [('Relu', {}), ('Erf', {'a': 0.7, 'b': 1.2, 'c': 0.1}), ('ABRelu', {'a': -0.4, 'b': 0.9}),
         ('Gelu', {}), ('Sin', {'a': 1.2, 'b': 0.8, 'c': 0.3}), ('Cos', {'a': 0.9, 'b': 1.1, 'c': -0.2}),
         ('Rbf', {'gamma': 0.5}), ('LeakyRelu', {'alpha': 0.1}), ('Abs', {}),
         ('Relu', {'do_stabilize': True}), ('Identity', {})]


def random_networks(count=40, seed=123):
    """Seeded random networks as layer specs [(name, kwargs)] that both the reference's stax
    and the oracle build alike: Dense stacks, or Conv stacks with filters of 1-3, strides,
    SAME / VALID / CIRCULAR padding and Avg / Sum / circular pools, each with a random
    activation and a Flatten / GlobalAvgPool / GlobalSumPool readout; x2 given or None."""
    rs = np.random.default_rng(seed)
    nets = []
    for _ in range(count):
        spec = []
        if rs.random() < 0.3:
            for _ in range(int(rs.integers(1, 4))):
                spec.append(('Dense', {'out_dim': 4, 'W_std': float(rs.uniform(0.8, 1.6)),
                                       'b_std': float(rs.uniform(0., 0.3))}))
                spec.append(_ACTS[int(rs.integers(len(_ACTS)))])
            shape = (int(rs.integers(5, 9)),)
        else:
            for _ in range(int(rs.integers(1, 3))):
                spec.append(('Conv', {
                    'out_chan': 1, 'filter_shape': (int(rs.integers(1, 4)), int(rs.integers(1, 4))),
                    'strides': (int(rs.integers(1, 3)), 1) if rs.random() < 0.3 else (1, 1),
                    'padding': ['SAME', 'VALID', 'CIRCULAR'][int(rs.integers(3))],
                    'W_std': float(rs.uniform(0.8, 1.6)), 'b_std': float(rs.uniform(0., 0.3))}))
                spec.append(_ACTS[int(rs.integers(len(_ACTS)))])
                if rs.random() < 0.4:
                    win = (int(rs.integers(1, 3)), int(rs.integers(1, 3)))
                    kind = int(rs.integers(3))
                    pad = ['SAME', 'VALID'][int(rs.integers(2))]
                    if kind == 0:
                        spec.append(('AvgPool', {'window_shape': win, 'strides': win, 'padding': pad,
                                                 'normalize_edges': bool(rs.random() < 0.5)}))
                    elif kind == 1:
                        spec.append(('SumPool', {'window_shape': win, 'strides': (1, 1),
                                                 'padding': pad}))
                    else:
                        spec.append(('AvgPool', {'window_shape': win, 'strides': (1, 1),
                                                 'padding': 'CIRCULAR'}))
            spec.append((['Flatten', 'GlobalAvgPool', 'GlobalSumPool'][int(rs.integers(3))], {}))
            shape = (int(rs.integers(5, 9)), int(rs.integers(5, 9)), 2)
        spec.append(('Dense', {'out_dim': 1, 'W_std': 1.2, 'b_std': 0.1}))
        x1 = rs.standard_normal((2,) + shape)
        x2 = rs.standard_normal((3,) + shape) if rs.random() < 0.7 else None
        nets.append((spec, x1, x2))
    return nets


def build(m, spec):
    return [getattr(m, name)(**kw) for name, kw in spec]


def _pred_net(m):
    return [m.Dense(64, 1.3, 0.1), m.Erf(), m.Dense(64, 1.2, 0.05), m.Relu(), m.Dense(2, 1.2, 0.05)]


PRED_TIMES = {'t_none': None, 't_inf': np.inf, 't_3': 3.0,
              't_array': np.array([[0.5, 2.], [10., 50.]])}
ENS_TIMES = {'t_none': None, 't_4': 4.0, 't_array': np.array([0.7, 30.])}


def prediction_inputs():
    rng = np.random.default_rng(77)
    return (rng.standard_normal((12, 6)), rng.standard_normal((5, 6)),
            rng.standard_normal((12, 2)), 0.1 * rng.standard_normal((12, 2)),
            0.1 * rng.standard_normal((5, 2)))


def jax_key():
    import jax
    return jax.random.PRNGKey(0)


def _load_reference(path):
    sys.path.insert(0, os.path.join(ROOT, 'oracle', 'jax_stand_in'))
    pkg = types.ModuleType('neural_tangents')
    pkg.__path__ = [os.path.join(path, 'neural_tangents')]  # its __init__ needs TF: skipped
    sys.modules['neural_tangents'] = pkg
    from neural_tangents import predict, stax
    return stax, predict


def main(path=DEFAULT_REFERENCE):
    stax, predict = _load_reference(path)
    sys.path.insert(0, HERE)
    import make_golden as G

    for name, (layers, gen, n1, get) in G.CASES.items():
        rng = np.random.default_rng(2024)
        x = gen(rng).astype(np.float32)
        x1, x2 = x[:n1], x[n1:]
        out = stax.serial(*layers(stax))[2](x1.astype(np.float64), x2.astype(np.float64), get)
        np.savez_compressed(os.path.join(HERE, f'{name}_reference.npz'), x1=x1, x2=x2,
                            **{g: np.asarray(v) for g, v in zip(get, out)})
        print(name, [np.asarray(v).shape for v in out])

    arrays = {}
    for name, (layers, _, _, get, kw) in KERNEL_CASES.items():
        x1, x2 = kernel_inputs(name)
        out = stax.serial(*layers(stax))[2](x1, x2, get, **kw)
        for g, v in zip(get, out):
            arrays[f'{name}/{g}'] = np.asarray(v)
        print(name, [np.asarray(v).shape for v in out])
    np.savez_compressed(os.path.join(HERE, 'reference_cases.npz'), **arrays)

    arrays = {}
    for i, (spec, x1, x2) in enumerate(random_networks()):
        kf = stax.serial(*build(stax, spec))[2]
        q, t = kf(x1, x2, ('nngp', 'ntk'))
        arrays[f'net{i}/nngp'] = np.asarray(q)
        arrays[f'net{i}/ntk'] = np.asarray(t)
        req = kf.input_req['diagonal_spatial']
        arrays[f'net{i}/diagonal_spatial_req'] = np.array([int(req.input), int(req.output)])
        init_fn = stax.serial(*build(stax, spec))[0]
        arrays[f'net{i}/out_shape'] = np.array(init_fn(jax_key(), x1.shape)[0])
        try:  # a diagonal-spatial request the network cannot serve
            kf(x1, x2, 'nngp', diagonal_spatial=True)
            msg = ''
        except ValueError as e:
            msg = str(e)
        arrays[f'net{i}/diagonal_spatial_error'] = np.array(msg)
    np.savez_compressed(os.path.join(HERE, 'reference_random.npz'), **arrays)
    print('random networks', len(arrays) // 2)

    xtr, xte, y, f0, g0 = prediction_inputs()
    kf = stax.serial(*_pred_net(stax))[2]
    kdd = kf(xtr, None, ('nngp', 'ntk'))
    ktd = kf(xte, xtr, ('nngp', 'ntk'))
    ktt = kf(xte, None, 'nngp')
    arrays = {'kernels/tt_nngp': np.asarray(ktt)}
    for g in ('nngp', 'ntk'):
        arrays[f'kernels/dd_{g}'] = np.asarray(getattr(kdd, g))
        arrays[f'kernels/td_{g}'] = np.asarray(getattr(ktd, g))
    for g in ('nngp', 'ntk'):
        pred = predict.gradient_descent_mse(np.asarray(getattr(kdd, g)), y, learning_rate=1.5,
                                            diag_reg=1e-3)
        for tn, t in PRED_TIMES.items():
            a, b = pred(t, f0, g0, np.asarray(getattr(ktd, g)))
            arrays[f'gd_{g}_{tn}/train'] = np.asarray(a)
            arrays[f'gd_{g}_{tn}/test'] = np.asarray(b)
    ens = predict.gradient_descent_mse_ensemble(kf, xtr, y, learning_rate=1.5, diag_reg=1e-3)
    for tn, t in ENS_TIMES.items():
        for g in ('nngp', 'ntk'):
            r = ens(t=t, x_test=xte, get=g, compute_cov=True)
            arrays[f'ens_{g}_{tn}/mean'] = np.asarray(r.mean)
            arrays[f'ens_{g}_{tn}/cov'] = np.asarray(r.covariance)
    gp = predict.gp_inference(kdd, y, diag_reg=1e-3)
    r = gp(get=('nngp', 'ntk'), k_test_train=ktd, k_test_test=ktt)
    for g, v in zip(('nngp', 'ntk'), r):
        arrays[f'gp_{g}/mean'] = np.asarray(v.mean)
        arrays[f'gp_{g}/cov'] = np.asarray(v.covariance)
    np.savez_compressed(os.path.join(HERE, 'reference_predictions.npz'), **arrays)
    print('predictions', len(arrays))


if __name__ == '__main__':
    main(*sys.argv[1:])
