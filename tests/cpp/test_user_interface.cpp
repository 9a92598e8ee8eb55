// The C++ facade used as the reference's tests use user_interface (test/test_python.cpp:8-31):
// 3D box 3.5^3, r = 0.4, seed 0; then throw_spheres in 2D.  Exit 0 on success.
#include <cmath>
#include <cstdio>

#include "rsa_gpu/user_interface.hxx"

int main() {
    constexpr int DIM = 3;
    user_interface::Point<DIM> l = {0., 0., 0.};
    user_interface::Point<DIM> L = {3.5, 3.5, 3.5};
    std::vector<std::tuple<double, double, int>> classes{{0.4, 1., 0}};
    user_interface::rsa_domain<DIM> domain(l, L, 0.4);
    user_interface::RadiusGenerator<DIM> rg(classes, domain.get_total_volume(), 0.);
    user_interface::rsa_algo<DIM> algo(domain, rg, 6000);
    algo.proceed(0);
    domain.domain_log();
    auto spheres = domain.extract_spheres();
    double vol = domain.compute_total_volume_of_spheres();
    std::printf("spheres %zu fraction %.4f\n", spheres.size(), vol / domain.get_total_volume());
    if (spheres.size() < 50 || spheres.size() > 75) return 1;
    auto s2 = user_interface::throw_spheres<2>({1., 1.}, {{0.01, 1., 3}}, 5, false);
    std::printf("2D discs %zu\n", s2.size());
    if (s2.size() < 1600 || s2.size() > 1900 || s2[0].phase != 3) return 2;
    try {
        user_interface::rsa_domain<2> bad({0., 0.}, {1., 1.}, 0.7);  // box smaller than 2 r: the reference throws
        return 3;
    } catch (const std::runtime_error&) {
    }
    // continuous radius law (test/test_random_radius_generator.cpp:13-29: r uniform in [0.05, 0.055])
    auto urg = user_interface::RadiusGenerator<DIM>::uniform(0.05, 0.055, 10000000000000000ull, 0);
    user_interface::rsa_domain<DIM> ud({0., 0., 0.}, {1., 1., 1.}, urg.get_max_radius());
    user_interface::rsa_algo<DIM> ualgo(ud, urg, 6000);
    ualgo.proceed(0);
    auto us = ud.extract_spheres();
    std::printf("uniform radii: spheres %zu\n", us.size());
    if (us.size() < 600 || us.size() > 760) return 4;
    for (const auto& s : us)
        if (s.radius < 0.05 || s.radius >= 0.055) return 5;
    // output files in the working directory: ParaviewOutput/rsa_mpi_0.pvtp and its piece
    ud.paraview();
    std::printf("paraview written\n");
    return 0;
}
