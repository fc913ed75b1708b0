"""Permissive ``simulacra.vis`` namespace (stub): every attribute is a dummy.

The reference's plotting modules read names from here at import time; plotting
itself is never exercised by the fixture generator.
"""


class _Dummy:
    def __init__(self, *args, **kwargs):
        pass

    def __call__(self, *args, **kwargs):
        return _Dummy()

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Dummy()

    def __iter__(self):
        return iter(())

    def __or__(self, other):
        return self

    def __ror__(self, other):
        return other


class Animator(_Dummy):
    pass


def __getattr__(name):
    if name.startswith("__"):
        raise AttributeError(name)
    return _Dummy()
