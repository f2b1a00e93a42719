"""The Kernel container of the analytic path (neural_tangents/_src/utils/kernel.py:27-149).

Arrays are torch float32 CUDA tensors in the reference's layout: a pair
kernel is [N1, N2, H, H', W, W'] (full spatial), [N1, N2, H, W] (diagonal
spatial) or [N1, N2] (no spatial axes); per-sample kernels drop N2. When
``is_reversed`` is set the spatial pairs appear in reversed order, exactly as
the reference returns them after an odd number of full-spatial Conv layers;
the kernels of this package always compute on the un-reversed order, which is
the same storage viewed through a permutation.
"""
from __future__ import annotations

import collections
import dataclasses
from typing import Optional

import torch


@dataclasses.dataclass
class Kernel:
    nngp: torch.Tensor
    ntk: Optional[torch.Tensor]
    cov1: torch.Tensor
    cov2: Optional[torch.Tensor]
    x1_is_x2: bool
    is_gaussian: bool
    is_reversed: bool
    is_input: bool
    diagonal_batch: bool
    diagonal_spatial: bool
    shape1: tuple
    shape2: tuple
    batch_axis: int = 0
    channel_axis: int = -1
    mask1: Optional[torch.Tensor] = None
    mask2: Optional[torch.Tensor] = None

    def replace(self, **kwargs) -> 'Kernel':
        return dataclasses.replace(self, **kwargs)

    def slice(self, n1_slice: slice, n2_slice: slice) -> 'Kernel':
        """kernel.py:151-167."""
        cov1 = self.cov1[n1_slice]
        cov2 = self.cov1[n2_slice] if self.cov2 is None else self.cov2[n2_slice]
        ntk = self.ntk
        return self.replace(
            cov1=cov1, nngp=self.nngp[n1_slice, n2_slice], cov2=cov2,
            ntk=ntk if ntk is None or ntk.ndim == 0 else ntk[n1_slice, n2_slice],
            shape1=(cov1.shape[0],) + tuple(self.shape1[1:]),
            shape2=(cov2.shape[0],) + tuple(self.shape2[1:]))

    def reverse(self) -> 'Kernel':
        """kernel.py:169-189: reverse the order of the spatial pairs."""
        return self.replace(cov1=reverse_zipped(self.cov1, 1), nngp=reverse_zipped(self.nngp, 2),
                            cov2=reverse_zipped(self.cov2, 1), ntk=reverse_zipped(self.ntk, 2),
                            is_reversed=not self.is_reversed)


def reverse_zipped(x: Optional[torch.Tensor], start: int) -> Optional[torch.Tensor]:
    """utils.py:465-480 as a permuted view."""
    if x is None or x.ndim <= start + 2:
        return x
    src = [j for i in range(x.ndim - 2, start - 1, -2) for j in (i, i + 1)]
    return x.permute(*range(start), *src)


def to_physical(x: Optional[torch.Tensor], start: int, reversed_: bool, diag: bool):
    """The un-reversed contiguous tensor the kernels compute on."""
    if x is None or x.ndim == 0:
        return x
    if reversed_ and not diag and x.ndim > start + 2:
        x = reverse_zipped(x, start)
    return x.contiguous()


def from_physical(x: Optional[torch.Tensor], start: int, reversed_: bool, diag: bool):
    if x is None or x.ndim == 0:
        return x
    if reversed_ and not diag and x.ndim > start + 2:
        return reverse_zipped(x, start)
    return x


_NAMEDTUPLES: dict = {}


def analytic_kernel(get: tuple, values: tuple):
    """The ``AnalyticKernel`` namedtuple the reference returns (utils.py:197-252)."""
    nt = _NAMEDTUPLES.get(get)
    if nt is None:
        nt = collections.namedtuple('AnalyticKernel', get)
        _NAMEDTUPLES[get] = nt
    return nt(*values)
