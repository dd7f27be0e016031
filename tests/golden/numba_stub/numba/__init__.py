"""Minimal stand-in for the ``numba`` package, used only to run the reference
python-bh CPU path (``implementations/sequential.py``) unmodified as plain
Python when generating golden vectors.  ``njit``/``jit`` become identity
decorators (they accept an optional signature and keyword options), ``prange``
is ``range``.  The arithmetic therefore runs as NumPy float64 scalar code,
which differs from Numba's ``fastmath=True`` build only at the ulp level.

Test infrastructure: nothing in the product imports this.
"""


def _identity(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def deco(fn):
        return fn

    return deco


njit = _identity
jit = _identity
guvectorize = _identity
vectorize = _identity
prange = range
float64 = float
int64 = int


class _Config:
    THREADING_LAYER = "omp"


config = _Config()


def threading_layer():
    return "omp"


class _Cuda:
    jit = staticmethod(_identity)

    @staticmethod
    def is_available():
        return False


cuda = _Cuda()
