"""Minimal stand-in for ``numba`` so that the unmodified reference package can be
imported in an environment without Numba (test infrastructure only).

``njit`` returns the Python function unchanged and ``prange`` is ``range``: the
arithmetic is the same IEEE float64 NumPy arithmetic Numba compiles without
fastmath; only speed and the random stream differ.
"""


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(func):
        return func

    return wrap


jit = njit
prange = range
