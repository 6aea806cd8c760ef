"""3-point Gauss-Legendre rule on [0, 1], pyminiweather/data/quadrature.py:4-74.

Held as read-only NumPy arrays (host constants; the initial-condition kernel
carries its own copy) behind read-only properties, so the singleton is
immutable as in the reference.
"""
import numpy as np


class GaussianQuadrature:
    def __init__(self):
        qpoints = np.array([0.112701665379258311482073460022, 0.500000000000000000000000000000,
                            0.887298334620741688517926539980], dtype=np.float64)
        qweights = np.array([0.277777777777777777777777777779, 0.444444444444444444444444444444,
                             0.277777777777777777777777777779], dtype=np.float64)
        gx, gz = np.meshgrid(qpoints, qpoints)
        wx, wz = np.meshgrid(qweights, qweights)
        arrays = dict(qpoints=qpoints, qweights=qweights, qweights_outer=np.outer(qweights, qweights),
                      qpoints_grid_x=gx, qpoints_grid_z=gz, qweights_grid_x=wx, qweights_grid_z=wz)
        for a in arrays.values():
            a.setflags(write=False)
        object.__setattr__(self, "_GaussianQuadrature__arrays", arrays)

    def __setattr__(self, name, value):
        raise AttributeError("Quadrature is immutable")

    @property
    def npoints(self):
        return 3

    @property
    def qpoints(self):
        return self.__arrays["qpoints"]

    @property
    def qweights(self):
        return self.__arrays["qweights"]

    @property
    def qweights_outer(self):
        return self.__arrays["qweights_outer"]

    @property
    def qpoints_grid_x(self):
        return self.__arrays["qpoints_grid_x"]

    @property
    def qpoints_grid_z(self):
        return self.__arrays["qpoints_grid_z"]

    @property
    def qweights_grid_x(self):
        return self.__arrays["qweights_grid_x"]

    @property
    def qweights_grid_z(self):
        return self.__arrays["qweights_grid_z"]


Quadrature = GaussianQuadrature()
