"""Host-side planning of the fused paths (no device needed): which networks the fused
whole-network kernel takes, which layer groups the differentiable path fuses, and the C ABI's
argument checks for the fused forward / backward entries."""
import ctypes
import math

import pytest
import torch


def _myrtle(s, depth=5, act=None):
    act = act or s.Relu
    f = {5: [2, 1, 1], 7: [2, 2, 2], 10: [3, 3, 3]}[depth]
    conv = lambda: s.Conv(1, (3, 3), padding='SAME', W_std=math.sqrt(2.), b_std=0.)
    layers = []
    for i, n in enumerate(f):
        for _ in range(n):
            layers += [conv(), act()]
        if i < 2:
            layers += [s.AvgPool((2, 2), (2, 2))]
    return layers + [s.GlobalAvgPool(), s.Dense(1, 1., 0.)]


@pytest.mark.parametrize('depth', [5, 7, 10])
def test_chain_plans_myrtle_family(depth):
    from nt_gb300 import _chain, stax
    kf = stax.serial(*_myrtle(stax, depth))[2]
    plan = _chain.plan_chain(kf.specs, (4, 32, 32, 3), False)
    assert plan is not None
    assert _chain.plan_chain(kf.specs, (4, 32, 32, 3), True) is None   # diagonal_spatial
    assert _chain.plan_chain(kf.specs, (4, 16, 16, 3), False) is None  # not 32 x 32


def test_chain_plans_every_dual_activation_but_not_do_stabilize():
    from nt_gb300 import _chain, stax
    for act in (lambda: stax.Gelu(), lambda: stax.Sin(1.1, 0.9, 0.2), lambda: stax.Rbf(0.5),
                lambda: stax.Erf(), lambda: stax.LeakyRelu(0.1)):
        kf = stax.serial(*_myrtle(stax, 5, act))[2]
        assert _chain.plan_chain(kf.specs, (2, 32, 32, 3), False) is not None
    kf = stax.serial(*_myrtle(stax, 5, lambda: stax.ABRelu(0., 1., do_stabilize=True)))[2]
    assert _chain.plan_chain(kf.specs, (2, 32, 32, 3), False) is None


def test_input_conv_act_fusion_choice():
    from nt_gb300 import _autograd, stax
    x = torch.empty((2, 32, 32, 3), device='meta')
    kf = stax.serial(*_myrtle(stax))[2]
    assert _autograd.input_conv_act_fusable(x, kf.specs, False)
    assert not _autograd.input_conv_act_fusable(x, kf.specs, True)
    assert not _autograd.input_conv_act_fusable(torch.empty((2, 32, 32, 5), device='meta'),
                                                kf.specs, False)
    assert not _autograd.input_conv_act_fusable(torch.empty((2, 16, 16, 3), device='meta'),
                                                kf.specs, False)
    w = torch.tensor(1.4, requires_grad=True)   # hyper-gradients take the layer-by-layer rules
    kw = stax.serial(stax.Conv(1, (3, 3), padding='SAME', W_std=w), stax.Relu())[2]
    assert not _autograd.input_conv_act_fusable(x, kw.specs, False)
    for layers in ([stax.Conv(1, (3, 3), padding='VALID'), stax.Relu()],
                   [stax.Conv(1, (3, 3), strides=(2, 2), padding='SAME'), stax.Relu()],
                   [stax.Conv(1, (3, 3), padding='SAME'), stax.Erf()],
                   [stax.Conv(1, (3, 3), padding='SAME', parameterization='standard'),
                    stax.Relu()]):
        assert not _autograd.input_conv_act_fusable(x, stax.serial(*layers)[2].specs, False)


def test_conv_act_and_act_pool_fusion_geometry():
    from nt_gb300 import _autograd, stax
    q = torch.empty((2, 3, 32, 32, 32, 32), device='meta')
    same3 = (3, 3, 1, 1, 1, 1, 32, 32, False, 2)
    assert _autograd.conv_act_fusable(q, same3)
    assert not _autograd.conv_act_fusable(q, (3, 3, 1, 1, 1, 1, 32, 32, True, 2))   # circular
    assert not _autograd.conv_act_fusable(q, (3, 3, 2, 2, 1, 1, 16, 16, False, 2))  # strided
    assert not _autograd.conv_act_fusable(torch.empty((2, 3, 16, 16, 16, 16), device='meta'),
                                          (3, 3, 1, 1, 1, 1, 16, 16, False, 2))
    pool = stax.AvgPool((2, 2), (2, 2))[2].specs[0]
    geom = _autograd._pool_geom(q, pool)
    assert _autograd.act_pool_fusable(q, geom)
    sump = stax.SumPool((2, 2), (2, 2))[2].specs[0]
    assert not _autograd.act_pool_fusable(q, _autograd._pool_geom(q, sump))
    q8 = torch.empty((2, 3, 8, 8, 8, 8), device='meta')
    assert _autograd.act_pool_fusable(q8, _autograd._pool_geom(q8, pool))
    q6 = torch.empty((2, 3, 6, 6, 6, 6), device='meta')
    assert not _autograd.act_pool_fusable(q6, _autograd._pool_geom(q6, pool))


def test_fused_entries_check_arguments_before_any_launch():
    """The fused forward / backward entries reject what their kernels do not cover, with an
    error code and message and without touching a device (the pointers are never read)."""
    from nt_gb300 import _lib as L
    lib = L.load()
    fake = 256
    act = L.Act(L.NTG_ACT_ABRELU, 0., 1., 0., 0, 0.)
    erf = L.Act(L.NTG_ACT_ERF, 1., 1., 0., 0, 0.)
    v = L.Var(fake, 1024, 32, 1)
    rc = lib.ntg_conv_act_bwd(None, fake, fake, fake, fake, 0, fake, None, 4, 2, 16, 2.0, act, v,
                              v, None, None)
    assert rc == 1 and b'32, 32, 32, 32' in lib.ntg_last_error()
    rc = lib.ntg_conv_act_bwd(None, fake, fake, fake, fake, 0, fake, None, 4, 2, 32, 2.0, erf, v,
                              v, None, None)
    assert rc == 1 and b'ABRelu' in lib.ntg_last_error()
    rc = lib.ntg_conv_act_bwd(None, fake + 4, fake, fake, fake, 0, fake, None, 4, 2, 32, 2.0, act,
                              v, v, None, None)
    assert rc == 1 and b'aligned' in lib.ntg_last_error()
    std = L.Affine(2.0, 0., 2.0, 0.5, 0., 0)   # not the NTK rule ntk = nngp + W^2 ntk_in
    rc = lib.ntg_input_conv_act_fs(None, fake, fake, 2, 2, 3, fake, fake, fake, std, act, v, v)
    assert rc == 1 and b'NTK rule' in lib.ntg_last_error()
    ntk = L.Affine(2.0, 0., 2.0, 1., 0., 1)
    rc = lib.ntg_input_conv_act_fs(None, fake, fake, 2, 2, 5, fake, fake, fake, ntk, act, v, v)
    assert rc == 1 and b'bad sizes' in lib.ntg_last_error()
    rc = lib.ntg_conv_act_pool_fs(None, fake, fake, fake, None, fake, fake, fake, fake, 4, 2, 32,
                                  ntk, act, v, v)
    assert rc == 1 and b'go together' in lib.ntg_last_error()
    rc = lib.ntg_input_ds(None, fake, None, 2, 3, 10, 3, fake)
    assert rc == 1 and b'go together' in lib.ntg_last_error()


def test_diagonal_spatial_request_rejected_for_pooled_readout():
    """stax_test.py:636-687: asking for diagonal_spatial=True from a network whose pooling needs
    the full spatial kernel raises ValueError before any kernel runs."""
    from nt_gb300 import stax
    kf = stax.serial(stax.Conv(1, (3, 3), padding='SAME'), stax.Relu(),
                     stax.AvgPool((2, 2), (2, 2)), stax.Flatten(), stax.Dense(1))[2]
    assert not bool(kf.diagonal)
    with pytest.raises(ValueError, match='diagonal_spatial'):
        kf(torch.zeros((2, 8, 8, 3)), None, 'nngp', diagonal_spatial=True)
    gap = stax.serial(stax.Conv(1, (3, 3), padding='SAME'), stax.Relu(), stax.GlobalAvgPool())[2]
    with pytest.raises(ValueError, match='diagonal_spatial'):
        gap(torch.zeros((2, 8, 8, 3)), None, 'nngp', diagonal_spatial=True)


def test_bench_step_credits_add_up_to_the_job():
    """bench.py credits each step of the symmetric job with the entries its tile produces; the
    210 tiles of the 2000 x 2000 triangle add up to the whole kernel."""
    import bench
    n = bench.N_SAMPLES // bench.TILE
    tiles = [(r, c) for r in range(n) for c in range(r, n)]
    assert len(tiles) == 210
    assert sum(bench.tile_entries(t) for t in tiles) == bench.N_SAMPLES ** 2


@pytest.mark.skipif(torch.cuda.is_available(), reason='checks the behaviour without a GPU')
def test_no_cpu_fallback():
    """Without a CUDA device the product path raises instead of computing on the host."""
    import numpy as np
    from nt_gb300 import stax
    kf = stax.serial(stax.Dense(4, 1.5, 0.05), stax.Relu(), stax.Dense(1))[2]
    with pytest.raises(RuntimeError, match='no CPU fallback'):
        kf(np.ones((2, 3), np.float32), None, 'nngp')


def test_diagonal_requirement_algebra():
    """tests/stax/requirements_test.py:116-132: composition of the diagonal requirements is
    associative (`>>` and `<<` alike, and they agree); `&` is commutative, associative and
    idempotent (requirements.py:432-515). For the product's `stax.Diagonal` and the oracle's."""
    import itertools
    from nt_gb300 import stax
    from oracle import nt_oracle as o
    for B, D in ((stax.Bool, stax.Diagonal), (o.Bool, o.Diagonal)):
        vals = [D(i, j) for i, j in itertools.product(B, repeat=2)]
        for a, b, c in itertools.product(vals, repeat=3):
            assert (a >> b) >> c == a >> (b >> c)
            if D is stax.Diagonal:
                assert c << (b << a) == (c << b) << a == (a >> b) >> c
                assert (a & b) == (b & a) and (a & b) & c == a & (b & c) and (a & a) == a
