"""Test-only stand-in for numba, used solely to import the reference package
when generating golden fixtures in a container without numba.

``njit``/``jit`` return the function unchanged (with or without keyword
arguments) and ``prange`` is ``range``, so the reference's kernels run as
plain Python with identical arithmetic.
"""


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(fn):
        return fn

    return wrap


jit = njit
prange = range


def get_num_threads():
    return 1


def set_num_threads(n):
    return None


def threading_layer():
    return "omp"
