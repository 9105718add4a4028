"""Stand-in for numba used only when the golden fixtures are generated.

The reference kernels are decorated with ``@njit(parallel=True, ...)`` and
loop with ``nb.prange``.  numba is not installed in the fixture container, so
this module turns ``njit``/``jit`` into identity decorators and ``prange`` into
``range``; the reference's own source then executes under NumPy with serial
loops and IEEE (non-fastmath) arithmetic.
"""


def _identity_decorator(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(fn):
        return fn

    return wrap


njit = _identity_decorator
jit = _identity_decorator
prange = range
