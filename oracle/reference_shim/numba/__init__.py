"""Identity stand-in for ``numba.njit`` (numba is not installed in this image).

Used only by ``tests/golden/make_golden.py`` to import the reference's pure
Python kernels (``solver/mac/kernels.py:3``) so that its outputs can be dumped
as golden fixtures.  JIT compilation does not change the arithmetic of those
loops (the reference keeps ``fastmath`` off), only their speed.
"""


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(fn):
        return fn
    return wrap


jit = njit
