"""Apps and the app factory (lbm/src/app/app.py, lbm/src/core/factory.py)."""
from .base_app import base_app
from .cavity import cavity
from .channel import turek, poiseuille, array, step, obstacle_array


class factory:
    def __init__(self):
        self.keys = {}

    def register(self, key, creator):
        self.keys[key] = creator

    def create(self, key, **kwargs):
        creator = self.keys.get(key)
        if not creator:
            raise ValueError(key)
        return creator(**kwargs)


app_factory = factory()
app_factory.register("cavity", cavity)
app_factory.register("turek", turek)
app_factory.register("poiseuille", poiseuille)
app_factory.register("array", array)
app_factory.register("step", step)
app_factory.register("obstacle_array", obstacle_array)
