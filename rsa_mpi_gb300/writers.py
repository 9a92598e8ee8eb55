"""Output files of the reference, written from sphere arrays copied off the GPU.

Formats follow the reference's writers byte for byte (numbers are printed like a
default-precision C++ ostream, 6 significant digits); the same spheres in the
same order give the same bytes:
  - ParaView .pvtp + .vtp pieces   include/operator_paraview.ixx:12-120
  - legacy VTK unstructured grid   include/rsa_data_storage.ixx:166-207 (write_spheres)
  - XYZ                            plugin/write_xyz.hpp:79-98
The reference lists spheres Real cell by Real cell (reference_order gives that
order for spheres extracted from the GPU; within one cell the GPU's order is
kept).  include/rsa_gpu/writers.hxx is the same set of writers in C++.
"""
from __future__ import annotations

import os

import numpy as np

_step = [0]


def _g(x) -> str:
    """operator<<(double) with the default precision 6."""
    s = f"{float(x):.6g}"
    return s


def reference_cell_keys(pos: np.ndarray, inf, sup, rad: float) -> np.ndarray:
    """Real-cell index of each centre in the reference's cell grid for a domain [inf, sup] of radius rad, one
    ghost layer: edge L_d / int(L_d / (2 rad)), shift inf_d - edge, x fastest (rsa_grid_traversal::define,
    rsa_grid_traversal.ixx:11-28; compute_cell_idx, :373-382)."""
    pos = np.asarray(pos, dtype=np.float64)
    key = np.zeros(len(pos), dtype=np.uint64)
    for d in reversed(range(pos.shape[1])):
        width = float(sup[d]) - float(inf[d])
        inside = int(width / (rad * 2))
        if inside == 0:
            raise RuntimeError("Too small domain wrt ghost layer")
        edge = width / inside
        shift = float(inf[d]) - 1 * edge
        ijk = ((pos[:, d] - shift) * (1.0 / edge)).astype(np.int64)  # truncation, as the int64 conversion
        key = key * np.uint64(inside + 2) + ijk.astype(np.uint64)
    return key


def reference_order(pos, rad, phase, inf, sup, rad_max):
    """The spheres reordered Real cell by Real cell as the reference lists them (apply_on_cells<Real> over
    build_real_traversal, rsa_grid_traversal.ixx:216-223); stable within a cell."""
    order = np.argsort(reference_cell_keys(pos, inf, sup, rad_max), kind="stable")
    return pos[order], rad[order], phase[order]


def write_paraview(a_name: str, pos: np.ndarray, rad: np.ndarray, phase: np.ndarray, rank: int = 0,
                   n_ranks: int = 1) -> str:
    """rsa_paraview::paraview: <a_name>/rsa_mpi_<step>.pvtp and
    <a_name>/rsa_mpi_<step>/rsa_mpi_<step>_<rank>.vtp; returns the .pvtp path."""
    step = _step[0]
    basename = "rsa_mpi"
    name = f"{basename}_{step}"
    directory = os.path.join(a_name, name)
    os.makedirs(directory, exist_ok=True)
    pvtp = os.path.join(a_name, name + ".pvtp")
    with open(pvtp, "w") as f:
        f.write(' <VTKFile type="PPolyData"> \n')
        f.write('   <PPolyData GhostLevel="0">\n')
        f.write('    <PPointData Scalar="id, tag">\n')
        f.write('      <PDataArray type="Int64" Name="Id"/>\n')
        f.write('      <PDataArray type="Int32" Name="Tag"/>\n')
        f.write('      <PDataArray type="Float64" Name="Radius"/>\n')
        f.write('    </PPointData>\n')
        f.write('     <PPoints>\n')
        f.write('       <PDataArray type="Float64" NumberOfComponents="3"/>\n')
        f.write('     </PPoints> \n')
        for i in range(n_ranks):
            f.write(f'     <Piece Source="{name}/{name}_{i}.vtp"/>\n')
        f.write('   </PPolyData>\n')
        f.write(' </VTKFile>\n')
    n = len(rad)
    dim = pos.shape[1] if n else 3
    xyz = np.zeros((n, 3))
    xyz[:, :min(dim, 3)] = pos[:, :min(dim, 3)]
    vtp = os.path.join(directory, f"{name}_{rank}.vtp")
    with open(vtp, "w") as f:
        f.write('<VTKFile type="PolyData">\n <PolyData>\n')
        f.write(f'   <Piece NumberOfPoints="{n}" NumberOfPolys="0">\n   <PointData>\n')
        f.write('     <DataArray type="Int64" Name="Id" format="ascii">\n')
        f.write("".join(f"{int(p)} " for p in phase) + "\n")
        f.write('     </DataArray>\n     <DataArray type="Int32" Name="Tag" format="ascii">\n')
        f.write("0 " * n + "\n")  # every extracted sphere is Validated (TypeTag 0)
        f.write('     </DataArray>\n     <DataArray type="Float64" Name="Radius" format="ascii">\n')
        f.write("".join(f"{_g(r)} " for r in rad) + "\n")
        f.write('     </DataArray>\n   </PointData>\n   <Points>\n')
        f.write('     <DataArray type="Float64" Name=""  NumberOfComponents="3" format="ascii">\n')
        f.write("".join(f"{_g(a)} {_g(b)} {_g(c)} " for a, b, c in xyz) + "\n")
        f.write('     </DataArray>\n   </Points>\n  </Piece>\n </PolyData>\n</VTKFile>\n')
    _step[0] += 1
    return pvtp


def write_vtk(path: str, pos: np.ndarray, rad: np.ndarray, phase: np.ndarray) -> None:
    """rsa_data_storage::write_spheres: legacy VTK, 2D and 3D only."""
    dim = pos.shape[1]
    if dim < 2 or dim > 3:
        raise RuntimeError("Not possible to vizualize in paraview!")
    n = len(rad)
    with open(path, "w") as f:
        f.write("# vtk DataFile Version 3.0\nSpheres\nASCII\nDATASET UNSTRUCTURED_GRID\n")
        f.write(f"POINTS {n} float\n")
        for p in pos:
            f.write(" ".join(_g(x) for x in p) + (" 0" if dim == 2 else "") + "\n")
        f.write(f"\nPOINT_DATA {n}\nSCALARS Id int 1\nLOOKUP_TABLE default\n")
        for ph in phase:
            f.write(f"{int(ph)}\n")
        f.write("\nSCALARS radius double 1\nLOOKUP_TABLE default\n")
        for r in rad:
            f.write(f"{_g(r)}\n")


def write_xyz(path: str, pos: np.ndarray, sup) -> None:
    """write_xyz (plugin/write_xyz.hpp:79-98): count, box, then "0 x y z" per sphere."""
    with open(path, "w") as f:
        f.write(f"{len(pos)}\n{_g(sup[0])} {_g(sup[1])} {_g(sup[2])}\n")
        for p in pos:
            f.write(f"0 {_g(p[0])} {_g(p[1])} {_g(p[2])}\n")
