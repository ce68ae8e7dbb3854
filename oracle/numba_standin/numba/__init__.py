"""Pure-Python stand-in for the ``numba`` package (oracle / fixture infrastructure only).

The reference package imports numba and, when it is present, routes its hot loops
through ``@njit`` kernels.  Numba is not installable in this image, and the
reference's NumPy fallback does not cover the default chain (``Cells._xi_deposit``
calls a kernel defined only under ``if _HAVE_NUMBA``).  Putting this directory first
on ``PYTHONPATH`` makes ``njit`` the identity decorator and ``prange`` the builtin
``range``, so the reference source runs UNMODIFIED (slowly) as plain Python.

Used only by ``tests/golden/make_fixtures.py`` to dump the reference's own binned
lens cells and outputs.  Never imported by the product package.
"""
__version__ = "0.0-standin"


def _decorator(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(fn):
        return fn
    return wrap


njit = _decorator
jit = _decorator
vectorize = _decorator
guvectorize = _decorator
prange = range


def set_num_threads(n):
    return None


def get_num_threads():
    return 1


class _Types:
    def __getattr__(self, name):
        return object


types = _Types()
