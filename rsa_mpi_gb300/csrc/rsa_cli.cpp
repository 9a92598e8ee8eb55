// rsa -- the reference's command-line sampler (command_line.cpp, include/rsa_parameters.hxx:77-187,
// include/rsa_test_perf.hxx:34-125) on the GPU, through the C++ facade include/rsa_gpu/user_interface.hxx.
//
//   rsa --dim D --radius r [--seed s] [--size n] [--n_draw k] [--inf x_0 .. x_{D-1}] [--sup y_0 .. y_{D-1}]
//       [--paraview 0|1] [--form 0|1]
//
// Same flags, defaults and checks as read_input: --dim first, unknown keys reported and skipped, the
// requirement messages printed (the reference then carries on: its `std::abort;` is never called).  One
// monodisperse run to maximality (algorithm::uniform_generate<DIM, 1>: radius r, volume fraction 1, nbshots
// = --size), then one line appended to outputFile.txt:
//   <ranks> <D> <r> <inf...> <sup...> <seed> <spheres> <seconds of the run> <seconds of the voxel check>
// with <ranks> = 1 and the voxel check not run (0.000000), as the reference's default.  --paraview 1 writes
// ParaviewOutput/ as rsa_paraview::paraview.  --n_draw only drives the reference's voxel-free method and is
// read and ignored, as there.  --form is not in the reference: 1 (default) the FP32 guard-band form, 0 every
// decision in FP64; both place the same spheres.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "rsa_gpu/user_interface.hxx"

namespace {

struct rsa_parameters {
    int DIM = -1;
    double radius = -1;
    std::vector<double> l_min = {0, 0, 0};
    std::vector<double> l_max = {1, 1, 1};
    int seed = 0;
    int n_draw = 10;
    int size = 6000;
    bool paraview = 0;
    int form = RSAGPU_FORM_FP32_GUARD;

    void display() const {
        std::cout << "============= Parameters =================" << std::endl;
        std::cout << "Dim         = " << DIM << std::endl;
        std::cout << "Radius      = " << radius << std::endl;
        std::cout << "Domain size = ";
        for (int d = 0; d < DIM - 1; d++) std::cout << "[" << l_min[d] << "," << l_max[d] << "]x";
        if (DIM >= 1) std::cout << "[" << l_min[DIM - 1] << "," << l_max[DIM - 1] << "]";
        std::cout << std::endl;
        std::cout << "Seed        = " << seed << std::endl;
        std::cout << "N Draw      = " << n_draw << std::endl;
        std::cout << "Size        = " << size << std::endl;
        std::cout << "Paraview    = " << paraview << " (0 disabled, 1 activated)" << std::endl;
        std::cout << "Form        = " << form << " (0 FP64, 1 FP32 guard band)" << std::endl;
        std::cout << "==========================================" << std::endl;
    }

    void minimal_requirement() const {
        if (DIM < 2) {
            std::cout << "DIM is not defined correctly, Value=" << DIM << "." << std::endl;
            std::cout << "Please use --dim Value." << std::endl;
        }
        if (radius < 0.0) {
            std::cout << "Radius is not defined correctly, Value=" << radius << "." << std::endl;
            std::cout << "Please use --radius Value." << std::endl;
        }
        if ((int)l_min.size() != DIM)
            std::cout << "Domain inf is not defined correctly, DIM= " << l_min.size() << " instead of " << DIM << "."
                      << std::endl;
        if ((int)l_max.size() != DIM)
            std::cout << "Domain inf is not defined correctly, DIM= " << l_min.size() << " instead of " << DIM << "."
                      << std::endl;
        for (int d = 0; d < DIM && d < (int)l_min.size() && d < (int)l_max.size(); d++)
            if (l_min[d] >= l_max[d])
                std::cout << "The domain simulation is not correctly defined, for DIM= " << d << " , inf >= max."
                          << std::endl;
    }
};

void help() {
    std::cout << "=== Available options ===" << std::endl;
    std::cout << "--dim [int, >= 2],           set dimension." << std::endl;
    std::cout << "--radius [double],           set sphere radius." << std::endl;
    std::cout << "--seed [int],                set seed used to generate random numbers." << std::endl;
    std::cout << "--size [int],                set the maximum number of spheres thrown per dart." << std::endl;
    std::cout << "--inf [double, ..., double], set the position of the bottom limit of the simulation domain." << std::endl;
    std::cout << "--sup [double, ..., double], set the position of the upper limit of the simulation domain." << std::endl;
    std::cout << "--paraview [int, 0 or 1],    disable [0] or activate [0] the feature: write paraview files, default is 0." << std::endl;
    std::cout << "--form [int, 0 or 1],        GPU arithmetic: 0 FP64, 1 FP32 with an FP64 guard band (default)." << std::endl;
}

// read_input (rsa_parameters.hxx:107-186)
rsa_parameters read_input(int argc, char** argv) {
    if (argc < 2) {
        std::cout << "Wrong number of arguments" << std::endl;
        help();
        std::exit(EXIT_FAILURE);
    }
    if (std::string(argv[1]) == "--help") {
        help();
        std::exit(EXIT_FAILURE);
    }
    rsa_parameters p;
    int i = 1;
    auto value = [&](int k) -> const char* {
        if (i + k >= argc) {
            std::cout << "Wrong number of arguments" << std::endl;
            std::abort();
        }
        return argv[i + k];
    };
    while (i < argc) {
        const std::string key = argv[i];
        if (i == 1 && key != "--dim") {
            std::cout << "Wrong arg: " << argv[i] << std::endl;
            std::cout << "Please, use the dimension input parameter as first input parameter (--dim)" << std::endl;
            std::abort();
        } else if (i == 1) {
            p.DIM = std::atoi(value(1));
            i += 2;
            p.l_min.assign(p.DIM > 0 ? p.DIM : 0, 0);
            p.l_max.assign(p.DIM > 0 ? p.DIM : 0, 0);
            continue;
        }
        if (key == "--radius") { p.radius = std::atof(value(1)); i += 2; continue; }
        if (key == "--seed") { p.seed = std::atoi(value(1)); i += 2; continue; }
        if (key == "--n_draw") { p.n_draw = std::atoi(value(1)); i += 2; continue; }
        if (key == "--size") { p.size = std::atoi(value(1)); i += 2; continue; }
        if (key == "--paraview") { p.paraview = std::atoi(value(1)); i += 2; continue; }
        if (key == "--form") { p.form = std::atoi(value(1)); i += 2; continue; }
        if (key == "--inf" || key == "--sup") {
            auto& v = key == "--inf" ? p.l_min : p.l_max;
            for (int d = 0; d < p.DIM; d++) v[d] = std::atof(value(1 + d));
            i += 1 + p.DIM;
            continue;
        }
        std::cout << key << " is ignored." << std::endl;
        i++;
    }
    p.minimal_requirement();
    return p;
}

template <class T>
void write_to_file(const std::string& path, T value) {
    std::ofstream f(path, std::ios::out | std::ios::app);
    if (f.is_open()) f << value;
}

// test_perf<DIM, 1> (rsa_test_perf.hxx:34-99) on the GPU
template <int DIM>
void test_perf(const rsa_parameters& p) {
    const std::string outputFile = "outputFile.txt";
    user_interface::Point<DIM> l_min{}, l_max{};
    for (int d = 0; d < DIM; d++) {
        l_min[d] = p.l_min[d];
        l_max[d] = p.l_max[d];
    }
    user_interface::rsa_domain<DIM> domain(l_min, l_max, p.radius);
    std::cout << " ==== log: domain [0] ==== " << std::endl;
    const auto start = std::chrono::system_clock::now();
    user_interface::RadiusGenerator<DIM> rg(std::vector<std::tuple<double, double, int>>{{p.radius, 1., 0}},
                                            domain.get_total_volume(), 0.);
    user_interface::rsa_algo<DIM> algo(domain, rg, p.size);
    algo.set_form(p.form);
    algo.proceed(static_cast<size_t>(p.seed));
    const auto end_algo = std::chrono::system_clock::now();
    const std::chrono::duration<double> seconds_for_algo = end_algo - start;
    const std::chrono::duration<double> seconds_for_vox = std::chrono::system_clock::now() - end_algo;
    uint64_t nb = 0;
    user_interface::detail::check(rsagpu_domain_count(domain.handle(), &nb));
    const int64_t total_nb_spheres = static_cast<int64_t>(nb);
    write_to_file(outputFile, 1);
    write_to_file(outputFile, " ");
    write_to_file(outputFile, DIM);
    write_to_file(outputFile, " ");
    write_to_file(outputFile, p.radius);
    write_to_file(outputFile, " ");
    for (int d = 0; d < DIM; d++) {
        write_to_file(outputFile, l_min[d]);
        write_to_file(outputFile, " ");
    }
    for (int d = 0; d < DIM; d++) {
        write_to_file(outputFile, l_max[d]);
        write_to_file(outputFile, " ");
    }
    write_to_file(outputFile, static_cast<size_t>(p.seed));
    write_to_file(outputFile, " ");
    write_to_file(outputFile, total_nb_spheres);
    write_to_file(outputFile, " ");
    write_to_file(outputFile, std::to_string(seconds_for_algo.count()));
    write_to_file(outputFile, " ");
    write_to_file(outputFile, std::to_string(seconds_for_vox.count()));
    write_to_file(outputFile, "\n");
    if (p.paraview) domain.paraview();
}

// test_perf_ dispatch (rsa_test_perf.hxx:101-112): the dimensions the GPU library is built for
void dispatch(const rsa_parameters& p) {
    switch (p.DIM) {
    case 2: return test_perf<2>(p);
    case 3: return test_perf<3>(p);
    case 4: return test_perf<4>(p);
    case 5: return test_perf<5>(p);
    case 6: return test_perf<6>(p);
    case 7: return test_perf<7>(p);
    default: throw std::runtime_error("Impossible!");
    }
}

}  // namespace

int main(int argc, char** argv) {
    rsa_parameters param = read_input(argc, argv);
    param.minimal_requirement();
    param.display();
    std::cout << "Number of openmp threads = 1\n" << std::endl;
    const auto start = std::chrono::system_clock::now();
    dispatch(param);
    const std::chrono::duration<double> elapsed = std::chrono::system_clock::now() - start;
    std::cout << "Time for 1 threads :  " << std::to_string(elapsed.count()) << "s" << std::endl;
    return EXIT_SUCCESS;
}
