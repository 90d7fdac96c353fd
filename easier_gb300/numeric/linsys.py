"""Linear system operator, easier/numeric/linsys.py:10-24."""
from torch import nn


class Linsys(nn.Module):
    """``A(x) = reducer(selector(x) * Ae) + x * Av``.

    On the per-op path this runs the gather and segmented-sum kernels; the
    fused solvers turn it into a SELL-32 matrix (``sparse.py``) once and
    run the fused SpMV instead.
    """

    def __init__(self, Av, Ae, selector, reducer) -> None:
        super().__init__()
        self.Av = Av
        self.Ae = Ae
        self.selector = selector
        self.reducer = reducer

    def forward(self, x):
        return self.reducer(self.selector(x) * self.Ae) + x * self.Av
