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


# ---------------------------------------------------------------------------
# Outputs of the reference itself (neural-tangents 0.6.6's own stax / predict code, run here on
# the numpy JAX stand-in by tests/golden/make_reference_golden.py): the oracle reproduces them.
# ---------------------------------------------------------------------------
_rspec = importlib.util.spec_from_file_location(
    'make_reference_golden', os.path.join(HERE, 'make_reference_golden.py'))
R = importlib.util.module_from_spec(_rspec)
_rspec.loader.exec_module(R)

REF_TOL = 1e-12  # relative to the largest entry; float64 on both sides


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize('name', sorted(G.CASES))
def test_oracle_matches_reference_fixture(name):
    layers, _, _, get = G.CASES[name]
    f = np.load(os.path.join(HERE, f'{name}_reference.npz'))
    out = o.serial(*layers(o))(f['x1'], f['x2'], get)
    for g, v in zip(get, out):
        assert _rel(v, f[g]) < REF_TOL, (g, _rel(v, f[g]))


@pytest.mark.parametrize('case', sorted(R.KERNEL_CASES))
def test_oracle_matches_reference_kernels(case):
    """Activations, paddings, strides, pools, readouts, full- and diagonal-spatial kernels.
    With x2 = None the NTK of a self pair (the diagonal) sits at correlation 1, where the
    ReLU rule's derivative term (pi - theta) / 2 pi with theta = atan2(sqrt(q11 q22 - q12^2),
    q12) turns the float64 rounding of q11 q22 - q12^2 (~1e-16) into theta ~ 1e-8: there the
    two implementations agree to 1e-7, everywhere else to REF_TOL."""
    layers, _, s2, get, kw = R.KERNEL_CASES[case]
    x1, x2 = R.kernel_inputs(case)
    ref = np.load(os.path.join(HERE, 'reference_cases.npz'))
    out = o.serial(*layers(o))(x1, x2, get, **kw)
    for g, v in zip(get, out):
        want = ref[f'{case}/{g}']
        assert np.shape(v) == want.shape, (g, np.shape(v), want.shape)
        if s2 is None and g == 'ntk':
            d = np.abs(np.asarray(v) - want) / np.abs(want).max()
            assert np.diag(d).max() < 1e-7
            assert (d - np.diag(np.diag(d))).max() < REF_TOL
        else:
            assert _rel(v, want) < REF_TOL, (g, _rel(v, want))


def test_oracle_matches_reference_on_random_networks():
    """Forty seeded random Dense / Conv networks (filters 1-3, strides, SAME / VALID /
    CIRCULAR padding, Avg / Sum / circular pools, all eleven activations, three readouts,
    x2 given or None): the oracle against the reference's outputs. Self-pair NTK entries of
    x2 = None kernels to 1e-7 (see test_oracle_matches_reference_kernels)."""
    ref = np.load(os.path.join(HERE, 'reference_random.npz'))
    for i, (spec, x1, x2) in enumerate(R.random_networks()):
        q, t = o.serial(*R.build(o, spec))(x1, x2, ('nngp', 'ntk'))
        assert _rel(q, ref[f'net{i}/nngp']) < REF_TOL, (i, spec)
        want = ref[f'net{i}/ntk']
        d = np.abs(np.asarray(t) - want) / max(np.abs(want).max(), 1e-300)
        if x2 is None:
            assert np.diag(d).max() < 1e-7, (i, spec)
            d = d - np.diag(np.diag(d))
        assert d.max() < REF_TOL, (i, spec, d.max())


def test_product_requirements_match_reference():
    """Host planning: for each random network the product's serial() derives the same
    diagonal_spatial requirement (requirements.py:401-515 folded over the layers) as the
    reference did, which decides the kernel layout every rule then runs on, and its init_fn
    the same output shape."""
    from nt_gb300 import stax
    ref = np.load(os.path.join(HERE, 'reference_random.npz'))
    for i, (spec, x1, _) in enumerate(R.random_networks()):
        init_fn, _, kernel_fn = stax.serial(*R.build(stax, spec))
        d = kernel_fn.input_req['diagonal_spatial']
        assert (int(d.input), int(d.output)) == tuple(ref[f'net{i}/diagonal_spatial_req']), \
            (i, spec)
        # and the same output shape from init_fn (padding, strides and pools alike)
        assert tuple(init_fn(0, x1.shape)[0]) == tuple(ref[f'net{i}/out_shape']), (i, spec)
        # a diagonal-spatial request the network cannot serve: the reference's ValueError,
        # word for word, raised before any kernel runs
        msg = str(ref[f'net{i}/diagonal_spatial_error'])
        if msg:
            with pytest.raises(ValueError) as err:
                kernel_fn(x1, None, 'nngp', diagonal_spatial=True)
            assert str(err.value) == msg, (i, str(err.value), msg)


def test_oracle_predictions_match_reference():
    """gradient_descent_mse (t = None, inf, a scalar, a 2 x 2 array of times),
    gradient_descent_mse_ensemble (t = None, a scalar, an array; means and covariances) and
    gp_inference, from the same kernel matrices as the reference's run."""
    P = np.load(os.path.join(HERE, 'reference_predictions.npz'))
    xtr, xte, y, f0, g0 = R.prediction_inputs()
    kdd = {g: P[f'kernels/dd_{g}'] for g in ('nngp', 'ntk')}
    ktd = {g: P[f'kernels/td_{g}'] for g in ('nngp', 'ntk')}
    ktt = P['kernels/tt_nngp']
    kf = o.serial(*R._pred_net(o))
    for g in ('nngp', 'ntk'):  # the kernels themselves (no self-pair NTK diagonal among them)
        assert _rel(kf(xte, xtr, g), ktd[g]) < REF_TOL
    assert _rel(kf(xtr, None, 'nngp'), kdd['nngp']) < REF_TOL
    for g in ('nngp', 'ntk'):
        pred = o.gradient_descent_mse(kdd[g], y, learning_rate=1.5, diag_reg=1e-3)
        for tn, t in R.PRED_TIMES.items():
            a, b = pred(t, f0, g0, ktd[g])
            assert _rel(a, P[f'gd_{g}_{tn}/train']) < 1e-11, (g, tn)
            assert _rel(b, P[f'gd_{g}_{tn}/test']) < 1e-11, (g, tn)

    def saved_kernels(a, b, get):  # the reference's kernel matrices for the three calls
        if b is None:
            return kdd[get] if a is xtr else ktt
        return ktd[get]

    ens = o.gradient_descent_mse_ensemble(saved_kernels, xtr, y, learning_rate=1.5,
                                          diag_reg=1e-3)
    for tn, t in R.ENS_TIMES.items():
        for g in ('nngp', 'ntk'):
            r = ens(t=t, x_test=xte, get=g, compute_cov=True)
            assert _rel(r.mean, P[f'ens_{g}_{tn}/mean']) < 1e-11, (g, tn)
            assert _rel(r.covariance, P[f'ens_{g}_{tn}/cov']) < 1e-11, (g, tn)
    gp = o.gp_inference(kdd, y, diag_reg=1e-3)(get=('nngp', 'ntk'), k_test_train=ktd,
                                                 k_test_test=ktt)
    for g, v in zip(('nngp', 'ntk'), gp):
        assert _rel(v.mean, P[f'gp_{g}/mean']) < 1e-11
        assert _rel(v.covariance, P[f'gp_{g}/cov']) < 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize('name', sorted(G.CASES))
def test_gpu_matches_reference_fixture(nt, name):
    """The CUDA path against the reference's own outputs on the fixtures' inputs."""
    layers, _, _, get = G.CASES[name]
    f = np.load(os.path.join(HERE, f'{name}_reference.npz'))
    out = nt.stax.serial(*layers(nt.stax))[2](f['x1'], f['x2'], get)
    for g, v in zip(get, out):
        got = v.detach().cpu().numpy()
        want = f[g]
        err = np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-30))
        assert err < 1e-5, (g, err)


# ---------------------------------------------------------------------------
# The stand-in's convolution and pooling, against direct loops: the primitives on which the
# reference's outputs above were computed (loaded under a private name, not as `jax`).
# ---------------------------------------------------------------------------
def _stand_in():
    import sys
    name = 'ntg_jax_stand_in'
    if name not in sys.modules:
        path = os.path.join(os.path.dirname(HERE), '..', 'oracle', 'jax_stand_in', 'jax')
        spec = importlib.util.spec_from_file_location(
            name, os.path.join(path, '__init__.py'), submodule_search_locations=[path])
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return sys.modules[name]


def _direct_conv_nchw(x, w, strides, pads, groups):
    n, c, h, wd = x.shape
    o_, i_, kh, kw = w.shape
    xp = np.pad(x, ((0, 0), (0, 0), pads[0], pads[1]))
    oh = (xp.shape[2] - kh) // strides[0] + 1
    ow = (xp.shape[3] - kw) // strides[1] + 1
    out = np.zeros((n, o_, oh, ow))
    per = o_ // groups
    for b in range(n):
        for oc in range(o_):
            g = oc // per
            for p in range(oh):
                for q in range(ow):
                    win = xp[b, g * i_:(g + 1) * i_, p * strides[0]:p * strides[0] + kh,
                             q * strides[1]:q * strides[1] + kw]
                    out[b, oc, p, q] = np.sum(win * w[oc])
    return out


@pytest.mark.parametrize('padding', ['SAME', 'VALID', ((1, 2), (0, 1))])
@pytest.mark.parametrize('strides', [(1, 1), (2, 1)])
def test_stand_in_convolution_is_lax_cross_correlation(padding, strides):
    """NCHW / OIHW and NHWC / HWIO layouts, feature groups, lax's SAME rule (output
    ceil(n / s), the smaller half of the padding first) and explicit padding."""
    lax = _stand_in().lax
    rng = np.random.default_rng(5)
    x = rng.standard_normal((2, 4, 7, 6))
    for groups in (1, 2):
        w = rng.standard_normal((4, 4 // groups, 3, 2))
        pads = lax.padtype_to_pads((7, 6), (3, 2), strides, padding)
        if padding == 'SAME':
            for n, k, s_, (lo, hi) in zip((7, 6), (3, 2), strides, pads):
                total = max((-(-n // s_) - 1) * s_ + k - n, 0)
                assert (lo, hi) == (total // 2, total - total // 2)
        want = _direct_conv_nchw(x, w, strides, pads, groups)
        got = lax.conv_general_dilated(x, w, strides, padding, feature_group_count=groups,
                                       dimension_numbers=('NCHW', 'OIHW', 'NCHW'))
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12)
        got = lax.conv_general_dilated(np.transpose(x, (0, 2, 3, 1)), np.transpose(w, (2, 3, 1, 0)),
                                       strides, padding, feature_group_count=groups,
                                       dimension_numbers=('NHWC', 'HWIO', 'NHWC'))
        np.testing.assert_allclose(np.transpose(got, (0, 3, 1, 2)), want, rtol=1e-12, atol=1e-12)


def test_stand_in_window_sums_and_dot_general():
    lax = _stand_in().lax
    rng = np.random.default_rng(6)
    x = rng.standard_normal((2, 5, 6, 3))
    got = lax.reduce_window(x, 0., lax.add, (1, 2, 3, 1), (1, 2, 1, 1), 'SAME')
    pads = lax.padtype_to_pads(x.shape, (1, 2, 3, 1), (1, 2, 1, 1), 'SAME')
    xp = np.pad(x, pads)
    want = np.zeros(got.shape)
    for i in range(got.shape[1]):
        for j in range(got.shape[2]):
            want[:, i, j, :] = xp[:, 2 * i:2 * i + 2, j:j + 3, :].sum(axis=(1, 2))
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12)
    a, b = rng.standard_normal((3, 4, 5)), rng.standard_normal((3, 5, 6))
    np.testing.assert_allclose(lax.dot_general(a, b, (((2,), (1,)), ((0,), (0,)))),
                               np.einsum('bij,bjk->bik', a, b), rtol=1e-12)
