// Writes the reference's output files with include/rsa_gpu/writers.hxx from a sphere file:
//   write_files <spheres.bin> <out_dir> <sup_0> .. <sup_{D-1}>
// spheres.bin: int32 dim, int64 n, double centres[n][dim], double radii[n], int32 phases[n].
// Output: <out_dir>/pv (ParaView), <out_dir>/spheres.vtk, and <out_dir>/spheres.xyz in 3D.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "rsa_gpu/writers.hxx"

template <int DIM>
int write_all(const std::vector<double>& c, const std::vector<double>& r, const std::vector<int>& ph,
              const std::string& dir, char** sup_arg) {
    std::array<double, DIM> sup{};
    for (int d = 0; d < DIM; d++) sup[d] = std::strtod(sup_arg[d], nullptr);
    rsa_gpu_output::paraview<DIM>(dir + "/pv", c.data(), r.data(), ph.data(), r.size());
    // the reference writes this file from grid.extract_data<Real>(), which leaves every phase 0
    const std::vector<int> zero(r.size(), 0);
    rsa_gpu_output::write_spheres<DIM>(dir + "/spheres.vtk", c.data(), r.data(), zero.data(), r.size());
    if constexpr (DIM >= 3) rsa_gpu_output::write_xyz<DIM>(dir + "/spheres.xyz", c.data(), r.size(), sup);
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    int32_t dim = 0;
    int64_t n = 0;
    if (std::fread(&dim, sizeof(dim), 1, f) != 1 || std::fread(&n, sizeof(n), 1, f) != 1) return 3;
    if (argc < 3 + dim) return 2;
    std::vector<double> c(n * dim), r(n);
    std::vector<int> ph(n);
    if (std::fread(c.data(), sizeof(double), c.size(), f) != c.size()) return 3;
    if (std::fread(r.data(), sizeof(double), r.size(), f) != r.size()) return 3;
    if (std::fread(ph.data(), sizeof(int), ph.size(), f) != ph.size()) return 3;
    std::fclose(f);
    switch (dim) {
    case 2: return write_all<2>(c, r, ph, argv[2], argv + 3);
    case 3: return write_all<3>(c, r, ph, argv[2], argv + 3);
    default: return 2;
    }
}
