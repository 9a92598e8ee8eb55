// user_interface.hxx -- C++ facade of the GB300 sampler with the reference's names and semantics
// (MarcJos/RSA_MPI include/user_interface.hxx:13-124), over the C ABI of include/rsagpu.h.
//
// Header-only; link with librsagpu.so.  Errors are thrown as std::runtime_error, as in the reference.
// Differences: the spheres live on the GPU of the calling thread.  extract_spheres() and paraview() list them
// Real cell by Real cell in the reference's cell-grid order (rsa_gpu_output::reference_cell_order); within
// one cell, spheres accepted in the same round can come in another order than the reference's.
#pragma once

#include <array>
#include <cstdint>
#include <functional>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "../rsagpu.h"
#include "writers.hxx"

namespace user_interface {

namespace detail {
inline void check(int code) {
    if (code != RSAGPU_OK) throw std::runtime_error(std::string("rsagpu: ") + rsagpu_last_error());
}
}  // namespace detail

template <int DIM>
using Point = std::array<double, DIM>;

// sac_de_billes::Sphere<DIM> (center, radius, phase)
template <int DIM>
struct rsa_sphere {
    Point<DIM> center{};
    double radius = 0;
    int phase = 0;
};

template <int DIM>
class rsa_domain {
public:
    // rsa_domain(global_inf, global_sup, a_rad) (user_interface.hxx:24-25)
    rsa_domain(const Point<DIM>& global_inf, const Point<DIM>& global_sup, const double a_rad)
        : inf_(global_inf), sup_(global_sup), rad_(a_rad) {
        rsagpu_domain* d = nullptr;
        detail::check(rsagpu_domain_create(DIM, inf_.data(), sup_.data(), a_rad, &d));
        ptr_ = std::shared_ptr<rsagpu_domain>(d, [](rsagpu_domain* p) { rsagpu_domain_destroy(p); });
    }
    const Point<DIM>& get_inf() const { return inf_; }
    const Point<DIM>& get_sup() const { return sup_; }
    double get_total_volume() const {
        double v = 0;
        detail::check(rsagpu_domain_total_volume(ptr_.get(), &v));
        return v;
    }
    double compute_total_volume_of_spheres() const {
        double v = 0;
        detail::check(rsagpu_domain_spheres_volume(ptr_.get(), &v));
        return v;
    }
    // domain_log (rsa_domain.ixx:151-162) as the reference prints it on one MPI rank: rank 0, the box, and
    // one send and one receive ghost buffer per neighbour direction of the periodic box (3^DIM - 1 each)
    void domain_log() const {
        int nbuf = 1;
        for (int d = 0; d < DIM; d++) nbuf *= 3;
        nbuf -= 1;
        auto write = [](const Point<DIM>& v) {
            for (int d = 0; d < DIM; d++) std::cout << (d ? "," : "") << v[d];
            std::cout << std::endl;
        };
        std::cout << " ==== log: domain [ 0 ] ==== " << std::endl;
        std::cout << " == m_inf : ";
        write(inf_);
        std::cout << " == m_sup : ";
        write(sup_);
        std::cout << " == sbuffer size :  " << nbuf << std::endl;
        std::cout << " == rbuffer size :  " << nbuf << std::endl;
        std::cout << " ================================== " << std::endl;
    }
    // extract_spheres (rsa_grid.ixx:88-98): the spheres in the reference's Real-cell order
    std::vector<rsa_sphere<DIM>> extract_spheres() const {
        std::vector<double> c, r;
        std::vector<int> ph;
        extract_arrays(c, r, ph);
        std::vector<rsa_sphere<DIM>> out(r.size());
        for (size_t i = 0; i < r.size(); i++) {
            for (int d = 0; d < DIM; d++) out[i].center[d] = c[i * DIM + d];
            out[i].radius = r[i];
            out[i].phase = ph[i];
        }
        return out;
    }
    // paraview() -> rsa_paraview::paraview(domain, "ParaviewOutput") (operator_paraview.hxx:35,
    // operator_paraview.ixx:69-120)
    void paraview() const {
        std::vector<double> c, r;
        std::vector<int> ph;
        extract_arrays(c, r, ph);
        rsa_gpu_output::paraview<DIM>("ParaviewOutput", c.data(), r.data(), ph.data(), r.size());
    }
    // centres (n x DIM), radii and phases copied off the GPU, in the reference's Real-cell order
    void extract_arrays(std::vector<double>& c, std::vector<double>& r, std::vector<int>& ph) const {
        uint64_t n = 0;
        detail::check(rsagpu_domain_extract(ptr_.get(), nullptr, nullptr, nullptr, 0, &n));
        std::vector<double> c0(n * DIM), r0(n);
        std::vector<int> ph0(n);
        detail::check(rsagpu_domain_extract(ptr_.get(), c0.data(), r0.data(), ph0.data(), n, &n));
        const auto order = rsa_gpu_output::reference_cell_order<DIM>(c0.data(), n, inf_, sup_, rad_);
        c.resize(n * DIM);
        r.resize(n);
        ph.resize(n);
        for (uint64_t i = 0; i < n; i++) {
            const size_t j = order[i];
            for (int d = 0; d < DIM; d++) c[i * DIM + d] = c0[j * DIM + d];
            r[i] = r0[j];
            ph[i] = ph0[j];
        }
    }
    rsagpu_domain* handle() const { return ptr_.get(); }

private:
    Point<DIM> inf_, sup_;
    double rad_;
    std::shared_ptr<rsagpu_domain> ptr_;
};

template <int DIM>
class RadiusGenerator {
public:
    // (radius, number, phase) classes (user_interface.hxx:64-66)
    RadiusGenerator(std::vector<std::tuple<double, uint64_t, int>> desired_radius_nb_phase, double exclusion_distance) {
        std::vector<double> r;
        std::vector<uint64_t> n;
        std::vector<int> p;
        for (auto& t : desired_radius_nb_phase) {
            r.push_back(std::get<0>(t));
            n.push_back(std::get<1>(t));
            p.push_back(std::get<2>(t));
        }
        rsagpu_radgen* g = nullptr;
        detail::check(rsagpu_radgen_create_counts(DIM, r.data(), n.data(), p.data(), (int)r.size(), exclusion_distance, &g));
        ptr_ = std::shared_ptr<rsagpu_radgen>(g, [](rsagpu_radgen* q) { rsagpu_radgen_destroy(q); });
    }
    // (radius, volume fraction, phase) classes (user_interface.hxx:71-74)
    RadiusGenerator(std::vector<std::tuple<double, double, int>> desired_radius_volumeFraction_phase, double volume,
                    double exclusion_distance) {
        std::vector<double> r, f;
        std::vector<int> p;
        for (auto& t : desired_radius_volumeFraction_phase) {
            r.push_back(std::get<0>(t));
            f.push_back(std::get<1>(t));
            p.push_back(std::get<2>(t));
        }
        rsagpu_radgen* g = nullptr;
        detail::check(rsagpu_radgen_create_fractions(DIM, r.data(), f.data(), p.data(), (int)r.size(), volume,
                                                     exclusion_distance, &g));
        ptr_ = std::shared_ptr<rsagpu_radgen>(g, [](rsagpu_radgen* q) { rsagpu_radgen_destroy(q); });
    }
    // continuous radius law r_min + (r_max - r_min) x, x uniform in [0, 1): the internal
    // sac_de_billes::RadiusGenerator<DIM>(min, max, &RandomRadiusGenerator(transform, phase), nb_spheres, 0)
    // with the uniform transform (radius_generator.ixx:39-48)
    static RadiusGenerator uniform(double r_min, double r_max, uint64_t nb_spheres, int phase) {
        rsagpu_radgen* g = nullptr;
        detail::check(rsagpu_radgen_create_uniform(DIM, r_min, r_max, nb_spheres, phase, &g));
        return RadiusGenerator(std::shared_ptr<rsagpu_radgen>(g, [](rsagpu_radgen* q) { rsagpu_radgen_destroy(q); }));
    }
    // sac_de_billes::RadiusGenerator<DIM>(min, max, &RandomRadiusGenerator(transform, phase), nb_spheres, 0)
    // (radius_generator.hxx:12-38) for any transform of x uniform in [0, 1): the transform is tabulated at
    // n_knots points x = j / (n_knots - 1) and the darts interpolate it linearly
    static RadiusGenerator random(std::function<double(double)> transform, uint64_t nb_spheres, int phase,
                                  int n_knots = 4097) {
        std::vector<double> t(n_knots);
        for (int j = 0; j < n_knots; j++) t[j] = transform(j / double(n_knots - 1));
        rsagpu_radgen* g = nullptr;
        detail::check(rsagpu_radgen_create_table(DIM, t.data(), n_knots, nb_spheres, phase, &g));
        return RadiusGenerator(std::shared_ptr<rsagpu_radgen>(g, [](rsagpu_radgen* q) { rsagpu_radgen_destroy(q); }));
    }
    double get_max_radius() const {
        double v = 0;
        detail::check(rsagpu_radgen_max_radius(ptr_.get(), &v));
        return v;
    }
    rsagpu_radgen* handle() const { return ptr_.get(); }

private:
    explicit RadiusGenerator(std::shared_ptr<rsagpu_radgen> p) : ptr_(std::move(p)) {}
    std::shared_ptr<rsagpu_radgen> ptr_;
};

template <int DIM>
class rsa_algo {
public:
    // (user_interface.hxx:95-97): keeps a reference to the domain, copies the radius generator
    rsa_algo(rsa_domain<DIM>& a_domain, RadiusGenerator<DIM>& a_radius_generator, int a_nbshots_singledraw)
        : domain_(&a_domain) {
        rsagpu_algo* a = nullptr;
        detail::check(rsagpu_algo_create(a_domain.handle(), a_radius_generator.handle(), a_nbshots_singledraw, &a));
        ptr_ = std::shared_ptr<rsagpu_algo>(a, [](rsagpu_algo* p) { rsagpu_algo_destroy(p); });
    }
    void proceed(size_t seed) { detail::check(rsagpu_algo_proceed(ptr_.get(), (uint64_t)seed)); }
    void reset_radius_generator(RadiusGenerator<DIM>& a_radius_generator) {
        detail::check(rsagpu_algo_reset_radgen(ptr_.get(), a_radius_generator.handle()));
    }
    // not in the reference: the arithmetic form (RSAGPU_FORM_FP64 or RSAGPU_FORM_FP32_GUARD) and schedule
    void set_form(int form, int schedule = RSAGPU_SCHEDULE_HEURISTIC) {
        detail::check(rsagpu_algo_set_form(ptr_.get(), form, schedule));
    }

private:
    rsa_domain<DIM>* domain_;
    std::shared_ptr<rsagpu_algo> ptr_;
};

// throw_spheres (user_interface.hxx:119-124 -> ::throw_spheres<DIM,1>, test.hxx:13-32): box [0, L], the radius
// generator built with volume 1 whatever L, domain radius = largest radius, 6000 shots per draw.
template <int DIM>
std::vector<rsa_sphere<DIM>> throw_spheres(Point<DIM> L,
                                           std::vector<std::tuple<double, double, int>> desired_radius_volumeFraction_phase,
                                           size_t seed, bool write_paraview) {
    Point<DIM> inf{};
    RadiusGenerator<DIM> rg(desired_radius_volumeFraction_phase, 1.0, 0.0);
    rsa_domain<DIM> domain(inf, L, rg.get_max_radius());
    {
        rsa_algo<DIM> algo(domain, rg, 6000);
        algo.proceed(seed);
    }
    if (write_paraview) domain.paraview();
    return domain.extract_spheres();
}

}  // namespace user_interface
