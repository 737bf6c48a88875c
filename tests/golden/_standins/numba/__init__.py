"""Inert stand-in for numba, used only to import the distance3d reference
with its JIT disabled (the same mode its own CI runs in) so that golden
vectors can be generated. ``njit`` returns the function unchanged; every
type expression (``numba.float64[::1]``, ``numba.types.Tuple(...)(...)``)
evaluates to an inert object.
"""


class _Inert:
    def __getattr__(self, name):
        return _Inert()

    def __getitem__(self, key):
        return _Inert()

    def __call__(self, *args, **kwargs):
        return _Inert()


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs and not isinstance(args[0], _Inert):
        return args[0]

    def deco(fn):
        return fn
    return deco


jit = njit


class _Typed:
    class Dict:
        @staticmethod
        def empty(*args, **kwargs):
            return {}


typed = _Typed()


def __getattr__(name):
    return _Inert()
