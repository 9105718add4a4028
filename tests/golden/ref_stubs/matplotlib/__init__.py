"""Headless stand-in for matplotlib used only by the golden-fixture generator.

Every attribute is a callable no-op object, so the reference's plotting calls
(``plt.imshow``, ``plt.savefig``, ``matplotlib.cm.ocean``...) do nothing.
"""
import sys
import types


class _Anything:
    def __call__(self, *args, **kwargs):
        return _Anything()

    def __getattr__(self, name):
        return _Anything()

    def __iter__(self):
        return iter((_Anything(), _Anything()))


class _Module(types.ModuleType):
    def __getattr__(self, name):
        return _Anything()


pyplot = _Module("matplotlib.pyplot")
cm = _Module("matplotlib.cm")
sys.modules["matplotlib.pyplot"] = pyplot
sys.modules["matplotlib.cm"] = cm


def __getattr__(name):
    return _Anything()
