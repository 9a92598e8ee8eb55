"""Drop-in replacement of the reference's Python module ``rsa_mpi_py``.

Same names, arguments and behaviour as Interface_python/Interface.cxx:22-120 of
the reference (pybind11 there, ctypes over the GPU library here):

    import rsa_mpi_gb300.rsa_mpi_py as rsa_mpi
    domain = rsa_mpi.rsa_domain_3D([0, 0, 0], [1, 1, 1], 0.05)
    rg = rsa_mpi.radius_generator_3D([[0.05, 0.25, 0], [0.025, 1, 0]], domain.get_total_volume(), 0.)
    algo = rsa_mpi.rsa_algo_3D(domain, rg, 6000)
    algo.proceed(0)
    spheres = domain.extract_spheres()

Errors the reference raises as std::runtime_error (RuntimeError in Python) are
raised as RsaGpuError, a RuntimeError.  Dimensions 2 to 7, as the reference's
module.  The GPU draws its own random stream (Philox), so a seed gives a
different sample from the reference's mt19937 stream, with the same
distribution.
"""
from __future__ import annotations

import sys

import numpy as np

from .sampler import Algo, Domain, RadiusGenerator
from . import writers


def set_nb_threads(nb_threads: int) -> None:
    """The reference sets the OpenMP thread count (Interface.cxx:22-31); the GPU library needs none."""
    sys.stderr.write(f"Number of openmp threads = {int(nb_threads)} (ignored: the sampler runs on the GPU)\n")


def _make(dim: int):
    dim_s = f"_{dim}D"

    class sphere:
        """Representation of sphere (Sphere<DIM>: center, radius, phase)."""

        __slots__ = ("center", "radius", "phase")

        def __init__(self, center=None, radius=0.0, phase=0):
            self.center = list(center) if center is not None else [0.0] * dim
            self.radius = float(radius)
            self.phase = int(phase)

        def __repr__(self):
            return f"sphere{dim_s}(center={self.center}, radius={self.radius}, phase={self.phase})"

    sphere.__name__ = sphere.__qualname__ = "sphere" + dim_s

    class rsa_domain:
        """Data storage for the spheres.  Pave a cuboid [l_min[0], l_max[0]] x ... [l_min[D-1], l_max[D-1]]."""

        def __init__(self, global_inf, global_sup, maximal_radius):
            if len(global_inf) != dim or len(global_sup) != dim:
                raise TypeError(f"rsa_domain{dim_s} expects {dim}-vectors")
            self._d = Domain(global_inf, global_sup, maximal_radius)

        def domain_log(self):
            print(f" ==== log: domain [0] ==== \n == m_inf : {list(self._d.inf)}\n == m_sup : {list(self._d.sup)}")

        def get_total_volume(self):
            """Return the total volume of the (global) cuboid."""
            return self._d.total_volume()

        def _ordered(self):
            d = self._d
            return writers.reference_order(*d.arrays(), d.inf, d.sup, d.rad_max)

        def paraview(self):
            """Print paraview output (rsa_paraview::paraview: a .pvtp and one .vtp)."""
            writers.write_paraview("ParaviewOutput", *self._ordered())

        def compute_total_volume_of_spheres(self):
            """Compute the cumulated volume of all spheres inside the whole domains."""
            return self._d.spheres_volume()

        def extract_spheres(self):
            """return list of spheres inside the domain"""
            pos, rad, ph = self._ordered()
            return [sphere(list(p), r, f) for p, r, f in zip(pos.tolist(), rad.tolist(), ph.tolist())]

        def extract_arrays(self):
            """The spheres as numpy arrays (centers [n, D], radii [n], phases [n]); not in the reference."""
            return self._d.arrays()

    rsa_domain.__name__ = rsa_domain.__qualname__ = "rsa_domain" + dim_s

    class radius_generator:
        """Store the prescribed radius distribution fixed by the user.

        radius_generator([[rad, N, phase], ...], exclusion_distance) or
        radius_generator([[rad, phi, phase], ...], volume_total, exclusion_distance).
        """

        def __init__(self, classes, *args):
            if len(args) == 1:
                self._rg = RadiusGenerator(dim, [(float(c[0]), int(c[1]), int(c[2])) for c in classes], None, args[0])
            elif len(args) == 2:
                self._rg = RadiusGenerator(dim, [(float(c[0]), float(c[1]), int(c[2])) for c in classes],
                                           float(args[0]), float(args[1]))
            else:
                raise TypeError("radius_generator(classes, exclusion) or (classes, volume, exclusion)")

    radius_generator.__name__ = radius_generator.__qualname__ = "radius_generator" + dim_s

    class rsa_algo:
        """Class for execution of the algorithm."""

        def __init__(self, domain, radgen, nbshots):
            self._domain = domain
            self._a = Algo(domain._d, radgen._rg, int(nbshots))

        def proceed(self, seed):
            """proceed(seed). Execute the RSA algorithm, with the seed for the pseudo-random generator."""
            self._a.proceed(int(seed))

        def reset_radius_generator(self, radgen):
            """Reset the radius generator, but retains the already placed spheres."""
            self._a.reset_radius_generator(radgen._rg)

    rsa_algo.__name__ = rsa_algo.__qualname__ = "rsa_algo" + dim_s

    def throw_spheres(L, desired_radius_volumeFraction_phase, seed, write_paraview):
        """([double, ...] L, [[double, double, int]] desired_radius_volumeFraction_phase, seed, write_paraview)

        Same as ::throw_spheres<DIM, 1> (include/test.hxx:13-32): box [0, L], the radius generator is built
        with volume 1 whatever L, domain radius = largest radius, 6000 shots per draw."""
        L = [float(x) for x in L]
        if len(L) != dim:
            raise TypeError(f"throw_spheres{dim_s} expects a {dim}-vector")
        classes = [(float(c[0]), float(c[1]), int(c[2])) for c in desired_radius_volumeFraction_phase]
        rg = RadiusGenerator(dim, classes, 1.0, 0.0)
        dom = Domain([0.0] * dim, L, rg.max_radius)
        algo = Algo(dom, rg, 6000)
        algo.proceed(int(seed))
        algo.close()
        pos, rad, ph = writers.reference_order(*dom.arrays(), dom.inf, dom.sup, dom.rad_max)
        if write_paraview:
            writers.write_paraview("ParaviewOutput", pos, rad, ph)
        out = [sphere(list(p), r, f) for p, r, f in zip(pos.tolist(), rad.tolist(), ph.tolist())]
        dom.close()
        return out

    throw_spheres.__name__ = "throw_spheres" + dim_s
    return sphere, rsa_domain, radius_generator, rsa_algo, throw_spheres


_mod = sys.modules[__name__]
for _dim in range(2, 8):
    for _obj in _make(_dim):
        setattr(_mod, _obj.__name__, _obj)
del _mod, _dim, _obj
