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
    return 0;
}
