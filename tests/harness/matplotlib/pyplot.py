"""matplotlib.pyplot stand-in (test infrastructure): figures are not drawn."""

from . import _Anything


def subplots(*args, **kwargs):
    return _Anything(), _Anything()


def __getattr__(name):
    return _Anything()
