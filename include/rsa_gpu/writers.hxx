// writers.hxx -- the reference's output files, written from spheres copied off the GPU:
//   ParaView .pvtp + one .vtp piece   rsa_paraview::paraview       (include/operator_paraview.ixx:12-120)
//   legacy VTK unstructured grid      rsa_data_storage::write_spheres (include/rsa_data_storage.ixx:166-207)
//   XYZ                               write_xyz                    (plugin/write_xyz.hpp:79-98)
//
// Numbers go through std::ostream with its default format (6 significant digits), as in the reference, so
// the same spheres in the same order give the same bytes.  The reference lists spheres Real cell by Real cell
// in its cell grid's traversal order; reference_cell_order gives that order for spheres extracted from the
// GPU (stable: within one cell the GPU's own order is kept, which can differ from the reference's order of
// spheres accepted in the same round).
//
// Header-only, no GPU needed: the functions take plain arrays (centres row-major n x DIM, radii, phases).
#pragma once

#include <array>
#include <cstddef>
#include <cstdint>
#include <filesystem>
#include <fstream>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>
#include <algorithm>

namespace rsa_gpu_output {

// Real-cell index of each centre in the reference's cell grid for a domain [inf, sup] of radius a_rad with one
// ghost layer: edge L_d / int(L_d / (2 a_rad)), shift inf_d - edge, x fastest (rsa_grid_traversal::define,
// rsa_grid_traversal.ixx:11-28; compute_cell_idx, :373-382).  Returns the stable permutation that sorts the
// spheres by that index (the order of apply_on_cells<Real> over build_real_traversal, :216-223).
template <int DIM>
std::vector<size_t> reference_cell_order(const double* centers, size_t n, const std::array<double, DIM>& inf,
                                         const std::array<double, DIM>& sup, double a_rad) {
    std::array<double, DIM> shift{}, inv{};
    std::array<uint64_t, DIM> cells{};
    for (int d = 0; d < DIM; d++) {
        const double length = a_rad * 2;
        const double width = sup[d] - inf[d];
        const int inside = static_cast<int>(width / length);
        if (inside == 0) throw std::runtime_error("Too small domain wrt ghost layer");
        const double edge = width / inside;
        inv[d] = 1. / edge;
        shift[d] = inf[d] - 1 * edge;
        cells[d] = static_cast<uint64_t>(inside + 2);
    }
    std::vector<uint64_t> key(n);
    for (size_t i = 0; i < n; i++) {
        uint64_t k = 0;
        for (int d = DIM - 1; d >= 0; d--) {
            const int64_t ijk = static_cast<int64_t>((centers[i * DIM + d] - shift[d]) * inv[d]);
            k = k * cells[d] + static_cast<uint64_t>(ijk);
        }
        key[i] = k;
    }
    std::vector<size_t> order(n);
    std::iota(order.begin(), order.end(), size_t{0});
    std::stable_sort(order.begin(), order.end(), [&key](size_t a, size_t b) { return key[a] < key[b]; });
    return order;
}

namespace detail {
inline int& paraview_step() {
    static int step = 0;  // rsa_paraview::step: one file set per call
    return step;
}

inline std::ofstream open_out(const std::string& name) {
    std::ofstream f(name);
    if (!f) throw std::runtime_error("cannot create the output file " + name);
    return f;
}
}  // namespace detail

// rsa_paraview::paraview(a_name, grid) on one rank: <a_name>/rsa_mpi_<step>.pvtp and
// <a_name>/rsa_mpi_<step>/rsa_mpi_<step>_0.vtp, every sphere tagged Validated (0).  Returns the .pvtp path.
// The reference prints three coordinates whatever DIM; for DIM < 3 it reads past the centre (undefined
// values), here the missing coordinates are written as 0.
template <int DIM>
std::string paraview(const std::string& a_name, const double* centers, const double* radii, const int* phases,
                     size_t n) {
    namespace fs = std::filesystem;
    const std::string basename = "rsa_mpi";
    const std::string name = basename + "_" + std::to_string(detail::paraview_step());
    const std::string directory = a_name + "/" + name;
    fs::create_directory(a_name);
    fs::create_directory(directory);
    const std::string pvtp = a_name + "/" + name + ".pvtp";
    {
        auto f = detail::open_out(pvtp);
        f << " <VTKFile type=\"PPolyData\"> " << std::endl;
        f << "   <PPolyData GhostLevel=\"0\">" << std::endl;
        f << "    <PPointData Scalar=\"id, tag\">" << std::endl;
        f << "      <PDataArray type=\"Int64\" Name=\"Id\"/>" << std::endl;
        f << "      <PDataArray type=\"Int32\" Name=\"Tag\"/>" << std::endl;
        f << "      <PDataArray type=\"Float64\" Name=\"Radius\"/>" << std::endl;
        f << "    </PPointData>" << std::endl;
        f << "     <PPoints>" << std::endl;
        f << "       <PDataArray type=\"Float64\" NumberOfComponents=\"3\"/>" << std::endl;
        f << "     </PPoints> " << std::endl;
        f << "     <Piece Source=\"" << name << "/" << name << "_0.vtp\"/>" << std::endl;
        f << "   </PPolyData>" << std::endl;
        f << " </VTKFile>" << std::endl;
    }
    auto f = detail::open_out(directory + "/" + name + "_0.vtp");
    f << "<VTKFile type=\"PolyData\">" << std::endl;
    f << " <PolyData>" << std::endl;
    f << "   <Piece NumberOfPoints=\"" << n << "\" NumberOfPolys=\"" << 0 << "\">" << std::endl;
    f << "   <PointData>" << std::endl;
    f << "     <DataArray type=\"Int64\" Name=\"Id\" format=\"ascii\">" << std::endl;
    for (size_t i = 0; i < n; i++) f << static_cast<uint64_t>(phases[i]) << " ";
    f << std::endl;
    f << "     </DataArray>" << std::endl;
    f << "     <DataArray type=\"Int32\" Name=\"Tag\" format=\"ascii\">" << std::endl;
    for (size_t i = 0; i < n; i++) f << 0 << " ";
    f << std::endl;
    f << "     </DataArray>" << std::endl;
    f << "     <DataArray type=\"Float64\" Name=\"Radius\" format=\"ascii\">" << std::endl;
    for (size_t i = 0; i < n; i++) f << radii[i] << " ";
    f << std::endl;
    f << "     </DataArray>" << std::endl;
    f << "   </PointData>" << std::endl;
    f << "   <Points>" << std::endl;
    f << "     <DataArray type=\"Float64\" Name=\"\"  NumberOfComponents=\"3\" format=\"ascii\">" << std::endl;
    for (size_t i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) f << (d < DIM ? centers[i * DIM + d] : 0.0) << " ";
    f << std::endl;
    f << "     </DataArray>" << std::endl;
    f << "   </Points>" << std::endl;
    f << "  </Piece>" << std::endl;
    f << " </PolyData>" << std::endl;
    f << "</VTKFile>" << std::endl;
    detail::paraview_step()++;
    return pvtp;
}

// rsa_data_storage::write_spheres: legacy VTK, DIM 2 and 3 only (a 0 appended to 2D points).
template <int DIM>
void write_spheres(const std::string& a_name, const double* centers, const double* radii, const int* phases,
                   size_t n) {
    if constexpr (DIM < 2 || DIM > 3) {
        throw std::runtime_error("Not possible to vizualize in paraview!");
    } else {
        auto f = detail::open_out(a_name);
        f << "# vtk DataFile Version 3.0" << std::endl;
        f << "Spheres" << std::endl;
        f << "ASCII" << std::endl;
        f << "DATASET UNSTRUCTURED_GRID" << std::endl;
        f << "POINTS " << n << " float" << std::endl;
        for (size_t i = 0; i < n; i++) {
            for (int d = 0; d < DIM; d++) {
                if (d) f << " ";
                f << centers[i * DIM + d];
            }
            if (DIM == 2) f << " 0";
            f << std::endl;
        }
        f << std::endl;
        f << "POINT_DATA " << n << std::endl;
        f << "SCALARS Id int 1" << std::endl;
        f << "LOOKUP_TABLE default" << std::endl;
        for (size_t i = 0; i < n; i++) f << static_cast<uint64_t>(phases[i]) << std::endl;
        f << std::endl;
        f << "SCALARS radius double 1" << std::endl;
        f << "LOOKUP_TABLE default" << std::endl;
        for (size_t i = 0; i < n; i++) f << radii[i] << std::endl;
    }
}

// write_xyz on one rank: the count, the first three components of the domain's upper corner, then
// "0 x y z" per sphere (type 0).  DIM >= 3: the reference reads past the arrays below that.
template <int DIM>
void write_xyz(const std::string& a_name, const double* centers, size_t n, const std::array<double, DIM>& a_sup) {
    static_assert(DIM >= 3, "write_xyz prints three coordinates");
    auto f = detail::open_out(a_name);
    f << n << std::endl;
    f << a_sup[0] << " " << a_sup[1] << " " << a_sup[2] << std::endl;
    for (size_t i = 0; i < n; i++)
        f << 0 << " " << centers[i * DIM] << " " << centers[i * DIM + 1] << " " << centers[i * DIM + 2]
          << std::endl;
}

}  // namespace rsa_gpu_output
