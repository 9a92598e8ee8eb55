/*
 * Driver for the REFERENCE sampler, compiled unmodified from its own headers
 * (MarcJos/RSA_MPI include/) against the single-rank MPI stand-in in
 * oracle/mpi_standin/.  TEST INFRASTRUCTURE ONLY: its outputs pin the oracle
 * restatement (oracle/rsa_oracle.c) and produce the committed golden fixtures.
 *
 * Usage:
 *   ref_rsa run <dim> <seed> <nbshots> <volume_mode> <L_0..L_{D-1}> <k> (<r> <phi> <phase>)*k  <out.bin>
 *
 *   volume_mode: 0 -> RadiusGenerator volume = total box volume
 *                     (rsa_algo::uniform_generate, operator_algorithm.ixx:507-515)
 *                1 -> volume = 1 (the quirk of ::throw_spheres, test.hxx:21)
 *
 * Runs algorithm::uniform_generate<DIM, 1, true> (operator_algorithm.ixx:517-524)
 * on the periodic box [0, L] with ghost layer 1 and domain radius = r_max, the
 * same call chain as ::throw_spheres (test.hxx:13-32).  The plog=true template
 * argument makes the reference print its per-round trace (miss rate, shots,
 * voxels) on stdout.  The final spheres are written to <out.bin>:
 *   int32 dim, int64 n, then n records of {double center[dim], double radius, int32 phase}.
 * The wall time of proceed() alone is printed as "proceed_seconds <t>".
 *
 *   ref_rsa runu <dim> <seed> <nbshots> <L_0..L_{D-1}> <r_min> <r_max> <count> <phase> <out.bin>
 *
 * The same run with a continuous radius law: sac_de_billes::RandomRadiusGenerator with the transform
 * x -> r_min + (r_max - r_min) x of a uniform x (radius_generator.hxx:12-38, the uniform law of
 * test/test_random_radius_generator.cpp:13-29), <count> spheres wanted.
 *
 *   ref_rsa reiter <dim> <seed> <nbshots> <L_0..L_{D-1}> <r_0> <multiplier> <steps> <out.bin>
 *
 * Re-iteration as scripts/main_max_frac.cpp:30-60: a maximal run with radius r_0, then <steps> times the
 * radius multiplied by <multiplier>, reset_radius_generator and proceed(seed) on the same domain
 * (rsa_algo::reset_radius_generator, operator_algorithm.ixx:238-250).
 *
 * With RSA_REF_OUTPUTS=<dir> in the environment, every mode also writes the reference's own output files of
 * the final spheres into <dir>: ParaView (rsa_paraview::paraview, operator_paraview.ixx:69-120) under <dir>/pv,
 * legacy VTK (rsa_data_storage::write_spheres of the Real cells' data, rsa_data_storage.ixx:166-207) as
 * <dir>/spheres.vtk and, in 3D, XYZ (plugin/write_xyz.hpp:79-98) as <dir>/spheres.xyz.
 */
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include <rsa_domain.hxx>
#include <radius_generator.hxx>
#include <operator_algorithm.hxx>
#include <operator_paraview.hxx>
#include <write_xyz.hpp>

namespace {

template<int DIM>
int run(int argc, char** argv) {
    // argv: run dim seed nbshots volume_mode L... k (r phi phase)* out
    int a = 2;
    size_t seed = std::strtoull(argv[a++], nullptr, 10);
    int nbshots = std::atoi(argv[a++]);
    int volume_mode = std::atoi(argv[a++]);
    std::array<double, DIM> inf{}, sup{};
    for (int d = 0; d < DIM; d++) {
        inf[d] = 0.;
        sup[d] = std::strtod(argv[a++], nullptr);
    }
    int k = std::atoi(argv[a++]);
    std::vector<std::tuple<double, double, int>> classes;
    for (int i = 0; i < k; i++) {
        double r = std::strtod(argv[a++], nullptr);
        double phi = std::strtod(argv[a++], nullptr);
        int ph = std::atoi(argv[a++]);
        classes.emplace_back(r, phi, ph);
    }
    std::string out = argv[a++];
    if (a > argc) return 2;

    double volume = 1.;
    for (int d = 0; d < DIM; d++) volume *= (sup[d] - inf[d]);
    if (volume_mode == 1) volume = 1.;
    sac_de_billes::RadiusGenerator<DIM> radius_generator(classes, volume);
    rsa_domain<DIM> domain(inf, sup, 1, radius_generator.get_max_radius());

    auto t0 = std::chrono::steady_clock::now();
    algorithm::uniform_generate<DIM, 1, true>(domain, radius_generator, nbshots, 10, seed);
    auto t1 = std::chrono::steady_clock::now();
    std::printf("proceed_seconds %.6f\n", std::chrono::duration<double>(t1 - t0).count());

    auto spheres = domain.extract_spheres();
    FILE* f = std::fopen(out.c_str(), "wb");
    if (!f) return 3;
    int32_t dim = DIM;
    int64_t n = spheres.size();
    std::fwrite(&dim, sizeof(dim), 1, f);
    std::fwrite(&n, sizeof(n), 1, f);
    for (const auto& s : spheres) {
        std::fwrite(s.center.data(), sizeof(double), DIM, f);
        double r = s.radius;
        int32_t ph = s.phase;
        std::fwrite(&r, sizeof(r), 1, f);
        std::fwrite(&ph, sizeof(ph), 1, f);
    }
    std::fclose(f);
    std::printf("spheres %lld volume_of_spheres %.17g\n", (long long)n,
        domain.compute_total_volume_of_spheres());
    if (const char* dir = std::getenv("RSA_REF_OUTPUTS")) {
        const std::string d = dir;
        rsa_paraview::paraview(domain, d + "/pv");
        auto data = domain.get_grid().template extract_data<TypeCell::Real>();
        data.write_spheres(d + "/spheres.vtk");
        if constexpr (DIM == 3) {
            auto sup = domain.get_sup();
            write_xyz<DIM>(d + "/spheres.xyz", data, sup);
        }
    }
    return 0;
}

template<int DIM>
int write_spheres(rsa_domain<DIM>& domain, const std::string& out) {
    auto spheres = domain.extract_spheres();
    FILE* f = std::fopen(out.c_str(), "wb");
    if (!f) return 3;
    int32_t dim = DIM;
    int64_t n = spheres.size();
    std::fwrite(&dim, sizeof(dim), 1, f);
    std::fwrite(&n, sizeof(n), 1, f);
    for (const auto& s : spheres) {
        std::fwrite(s.center.data(), sizeof(double), DIM, f);
        double r = s.radius;
        int32_t ph = s.phase;
        std::fwrite(&r, sizeof(r), 1, f);
        std::fwrite(&ph, sizeof(ph), 1, f);
    }
    std::fclose(f);
    std::printf("spheres %lld volume_of_spheres %.17g\n", (long long)n,
        domain.compute_total_volume_of_spheres());
    if (const char* dir = std::getenv("RSA_REF_OUTPUTS")) {
        const std::string d = dir;
        rsa_paraview::paraview(domain, d + "/pv");
        auto data = domain.get_grid().template extract_data<TypeCell::Real>();
        data.write_spheres(d + "/spheres.vtk");
        if constexpr (DIM == 3) {
            auto sup = domain.get_sup();
            write_xyz<DIM>(d + "/spheres.xyz", data, sup);
        }
    }
    return 0;
}

template<int DIM>
int run_uniform_radius(int argc, char** argv) {
    // argv: runu dim seed nbshots L... r_min r_max count phase out
    int a = 2;
    size_t seed = std::strtoull(argv[a++], nullptr, 10);
    int nbshots = std::atoi(argv[a++]);
    std::array<double, DIM> inf{}, sup{};
    for (int d = 0; d < DIM; d++) {
        inf[d] = 0.;
        sup[d] = std::strtod(argv[a++], nullptr);
    }
    const double r_min = std::strtod(argv[a++], nullptr);
    const double r_max = std::strtod(argv[a++], nullptr);
    const uint64_t count = std::strtoull(argv[a++], nullptr, 10);
    const uint64_t phase = std::strtoull(argv[a++], nullptr, 10);
    std::string out = argv[a++];
    if (a > argc) return 2;
    auto transform = [r_min, r_max](double x) { return r_min + (r_max - r_min) * x; };
    sac_de_billes::RandomRadiusGenerator random_radius(transform, phase);
    sac_de_billes::RadiusGenerator<DIM> radius_generator(r_min, r_max, &random_radius, count, 0.);
    rsa_domain<DIM> domain(inf, sup, 1, radius_generator.get_max_radius());
    auto t0 = std::chrono::steady_clock::now();
    algorithm::uniform_generate<DIM, 1, true>(domain, radius_generator, nbshots, 10, seed);
    auto t1 = std::chrono::steady_clock::now();
    std::printf("proceed_seconds %.6f\n", std::chrono::duration<double>(t1 - t0).count());
    return write_spheres<DIM>(domain, out);
}

template<int DIM>
int run_reiterate(int argc, char** argv) {
    // argv: reiter dim seed nbshots L... r0 multiplier steps out
    int a = 2;
    size_t seed = std::strtoull(argv[a++], nullptr, 10);
    int nbshots = std::atoi(argv[a++]);
    std::array<double, DIM> inf{}, sup{};
    for (int d = 0; d < DIM; d++) {
        inf[d] = 0.;
        sup[d] = std::strtod(argv[a++], nullptr);
    }
    double rad = std::strtod(argv[a++], nullptr);
    const double multiplier = std::strtod(argv[a++], nullptr);
    const int steps = std::atoi(argv[a++]);
    std::string out = argv[a++];
    if (a > argc) return 2;
    double volume = 1.;
    for (int d = 0; d < DIM; d++) volume *= (sup[d] - inf[d]);
    sac_de_billes::RadiusGenerator<DIM> radius_generator(
        std::vector<std::tuple<double, double, int>>{{rad, 1., 0}}, volume);
    rsa_domain<DIM> domain(inf, sup, 1, radius_generator.get_max_radius());
    algorithm::rsa_algo<DIM> algo(domain, radius_generator, nbshots, 10);
    auto t0 = std::chrono::steady_clock::now();
    algo.template proceed<1>(seed);
    for (int j = 0; j < steps; j++) {
        rad *= multiplier;
        sac_de_billes::RadiusGenerator<DIM> next(std::vector<std::tuple<double, double, int>>{{rad, 1., 0}}, volume);
        algo.reset_radius_generator(next);
        algo.template proceed<1>(seed);
    }
    auto t1 = std::chrono::steady_clock::now();
    std::printf("proceed_seconds %.6f\n", std::chrono::duration<double>(t1 - t0).count());
    return write_spheres<DIM>(domain, out);
}

} // namespace

int main(int argc, char** argv) {
    if (argc >= 3 && std::string(argv[1]) == "reiter") {
        int dim = std::atoi(argv[2]);
        argv[2] = argv[1];
        argv++;
        argc--;
        switch (dim) {
        case 2: return run_reiterate<2>(argc, argv);
        case 3: return run_reiterate<3>(argc, argv);
        default:
            std::fprintf(stderr, "dim %d not built\n", dim);
            return 2;
        }
    }
    if (argc >= 3 && std::string(argv[1]) == "runu") {
        int dim = std::atoi(argv[2]);
        argv[2] = argv[1];
        argv++;
        argc--;
        switch (dim) {
        case 2: return run_uniform_radius<2>(argc, argv);
        case 3: return run_uniform_radius<3>(argc, argv);
        default:
            std::fprintf(stderr, "dim %d not built\n", dim);
            return 2;
        }
    }
    if (argc < 3 || std::string(argv[1]) != "run") {
        std::fprintf(stderr, "usage: ref_rsa run <dim> <seed> <nbshots> <volume_mode> <L...> <k> (<r> <phi> <phase>)* <out>\n");
        return 2;
    }
    int dim = std::atoi(argv[2]);
    // shift argv so that argv[2] is the seed
    argv[2] = argv[1];
    argv++;
    argc--;
    switch (dim) {
    case 2: return run<2>(argc, argv);
    case 3: return run<3>(argc, argv);
    case 4: return run<4>(argc, argv);
    default:
        std::fprintf(stderr, "dim %d not built\n", dim);
        return 2;
    }
}
