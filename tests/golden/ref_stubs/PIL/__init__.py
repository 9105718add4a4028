"""Headless stand-in for PIL used only by the golden-fixture generator."""
import sys
import types


class _Anything:
    def __call__(self, *args, **kwargs):
        return _Anything()

    def __getattr__(self, name):
        return _Anything()


class _Module(types.ModuleType):
    def __getattr__(self, name):
        return _Anything()


Image = _Module("PIL.Image")
ImageChops = _Module("PIL.ImageChops")
sys.modules["PIL.Image"] = Image
sys.modules["PIL.ImageChops"] = ImageChops
