"""GB300 sampler of maximal Poisson-sphere packings (random sequential addition with voxel
subdivision), a drop-in for the hot path of MarcJos/RSA_MPI.

  rsa_mpi_gb300.rsa_mpi_py   the reference's Python module (rsa_domain_3D, radius_generator_3D, ...)
  rsa_mpi_gb300.sampler      Domain / RadiusGenerator / Algo classes over the C ABI
  include/rsagpu.h           the C ABI (librsagpu.so, built by rsa_mpi_gb300.build)
"""
from ._lib import RsaGpuError  # noqa: F401
