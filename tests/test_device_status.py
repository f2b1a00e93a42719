"""The device error words reach the caller as NtgError (host logic; no GPU).

Kernels with bounded pipeline waits set a device error word when a wait runs
out. The public calls (kernel_fn, nt.batch, their backward passes, a captured
batch) read the words once at their outermost level through
_lib.check_device; these tests replace the library with a fake whose
ntg_device_status reports a timeout, so nothing runs on a device.
"""
import pytest
import torch


class _FakeLib:
    def __init__(self, code):
        self.code, self.reads = code, 0

    def ntg_device_status(self):
        self.reads += 1
        return self.code

    def ntg_last_error(self):
        return b'a bounded device wait ran out in a streamed kernel'


class _Stream:
    def synchronize(self):
        pass


@pytest.fixture
def fake_device(monkeypatch):
    import nt_gb300  # noqa: F401  (no library load: the fake stands in for it)
    from nt_gb300 import _lib as L

    def install(code):
        fake = _FakeLib(code)
        monkeypatch.setattr(L, 'load', lambda: fake)
        monkeypatch.setattr(torch.cuda, 'is_available', lambda: True)
        monkeypatch.setattr(torch.cuda, 'current_stream', lambda *a, **k: _Stream())
        return fake
    return install


def test_check_device_raises_on_timeout_word(fake_device):
    from nt_gb300 import _lib as L
    fake_device(5)
    with pytest.raises(L.NtgError, match='wait timeout'):
        L.check_device('kernel_fn')


def test_check_device_passes_on_zero_word(fake_device):
    from nt_gb300 import _lib as L
    fake = fake_device(0)
    L.check_device('kernel_fn')
    assert fake.reads == 1


def test_boundary_checks_once_at_the_outermost_level(fake_device):
    from nt_gb300 import _lib as L
    fake = fake_device(0)
    with L.boundary('nt.batch'):
        for _ in range(3):  # per-tile kernel_fn calls inside a batch
            with L.boundary('kernel_fn'):
                pass
        assert fake.reads == 0
    assert fake.reads == 1


def test_boundary_raises_after_the_public_call(fake_device):
    from nt_gb300 import _lib as L
    fake_device(5)
    ran = []
    with pytest.raises(L.NtgError, match='nt.batch'):
        with L.boundary('nt.batch'):
            ran.append(1)
    assert ran == [1]


def test_boundary_does_not_mask_the_call_own_exception(fake_device):
    from nt_gb300 import _lib as L
    fake = fake_device(5)
    with pytest.raises(ValueError):
        with L.boundary('kernel_fn'):
            raise ValueError('bad argument')
    assert fake.reads == 0


def test_kernel_fn_raises_when_the_device_word_is_set(fake_device, monkeypatch):
    """The public kernel_fn reads the words after its rules ran (the rules are stubbed)."""
    from nt_gb300 import _lib as L, stax
    fake_device(5)
    kf = stax.serial(stax.Dense(1), stax.Relu())[2]
    monkeypatch.setattr(type(kf), '_call', lambda self, *a, **k: 'kernels')
    with pytest.raises(L.NtgError, match='kernel_fn: wait timeout'):
        kf(None, None, 'nngp')


def test_batch_raises_when_the_device_word_is_set(fake_device, monkeypatch):
    import nt_gb300 as nt
    from nt_gb300 import _lib as L, stax
    fake_device(5)
    kf = stax.serial(stax.Dense(1), stax.Relu())[2]
    monkeypatch.setattr(type(kf), '_call', lambda self, *a, **k: 'kernels')
    from nt_gb300.kernel import Kernel
    k = Kernel.__new__(Kernel)
    with pytest.raises(L.NtgError, match='nt.batch: wait timeout'):
        nt.batch(kf, 10)(k)
