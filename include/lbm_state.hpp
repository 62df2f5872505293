// lbm_state.hpp — C++ host mirror of taktoa/chemsim's src/lbm.rs surface over
// the C ABI of liblbm_cuda.so (lbm_cuda.h).  Header-only; link with
// -llbm_cuda.
//
// Names, argument meaning and error behaviour follow lbm.rs:
//   Discretization            src/lbm.rs:75-86
//   D2Q9::directions          src/lbm.rs:202-282
//   compute_equilibrium       src/lbm.rs:43-71
//   BGK, TRT                  src/lbm.rs:345-451
//   State<L>::initial / step / size / delta_x / delta_t / populations /
//   isothermal_speed_of_sound / density / pressure / momentum_density /
//   velocity / speed / equilibrium / non_equilibrium / is_unstable /
//   geometry               src/lbm.rs:670-819
// Fields are row-major y * w + x vectors (the layout of Matrix::new /
// get_underlying); populations are 9 such planes in D2Q9 direction order.
// Where lbm.rs panics (assert!), this header throws std::logic_error; a
// negative status of the C ABI throws std::runtime_error with the library's
// message.  The stepping runs on the GPU (one fused launch per step).
#pragma once

#include <cmath>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "lbm_cuda.h"

namespace chemsim {

using Scalar = float;
using Field = std::vector<float>;

inline void check(int status) {
    if (status != LBM_OK)
        throw std::runtime_error("lbm-cuda status " + std::to_string(status) + ": " +
                                 lbm_last_error_string());
}

inline void require(bool ok, const char* what) {
    if (!ok) throw std::logic_error(what);
}

// src/lbm.rs:75-86
struct Discretization {
    Scalar delta_x = 1.f;
    Scalar delta_t = 1.f;
    Scalar isothermal_speed_of_sound() const { return delta_x / (std::sqrt(3.0f) * delta_t); }
};

// src/lbm.rs:90-95, 202-282 (weights and velocities; the stencils are the
// kernel's business)
struct Direction {
    Scalar w_scalar;
    int cx, cy;
};

struct D2Q9 {
    // src/lbm.rs:187-200: nine planes of one size
    D2Q9(std::vector<Field> populations, int w, int h)
        : pops(std::move(populations)), w_(w), h_(h) {
        require(pops.size() == 9, "D2Q9 needs 9 populations");
        for (const auto& p : pops)
            require(p.size() == size_t(w) * size_t(h), "population shapes differ");
    }
    static std::vector<Direction> directions() {
        return {{16.f / 36.f, 0, 0}, {4.f / 36.f, 1, 0},  {4.f / 36.f, 0, 1},
                {4.f / 36.f, -1, 0}, {4.f / 36.f, 0, -1}, {1.f / 36.f, 1, 1},
                {1.f / 36.f, -1, 1}, {1.f / 36.f, -1, -1}, {1.f / 36.f, 1, -1}};
    }
    std::pair<int, int> size() const { return {w_, h_}; }
    std::vector<Field> pops;

  private:
    int w_, h_;
};

// src/lbm.rs:345-370
struct BGK {
    Scalar tau;
    Scalar kinematic_shear_viscosity(const Discretization& d) const {
        return (d.delta_x * d.delta_x / (3.f * d.delta_t * d.delta_t)) * (tau - d.delta_t / 2.f);
    }
};

// src/lbm.rs:374-451
struct TRT {
    Scalar tau_minus, tau_plus;
    static TRT create(Scalar lambda, Scalar ks_viscosity, const Discretization& d) {
        const Scalar cs = d.isothermal_speed_of_sound();
        const Scalar tp = d.delta_t * ((ks_viscosity / (cs * cs)) + 0.5f);
        const Scalar tm = d.delta_t * ((lambda / ((tp / d.delta_t) - 0.5f)) + 0.5f);
        return {tm, tp};
    }
    Scalar kinematic_shear_viscosity(const Discretization& d) const {
        const Scalar cs = d.isothermal_speed_of_sound();
        return cs * cs * (tau_plus / d.delta_t - 0.5f);
    }
};

// A device-resident lattice handle (RAII over lbm_create / lbm_destroy).
class Lattice {
  public:
    Lattice(int w, int h, Scalar tau, int precision = LBM_F32, int flags = LBM_REFERENCE_FLAGS)
        : w_(w), h_(h) {
        lbm_lattice* raw = nullptr;
        check(lbm_create(w, h, tau, precision, flags, &raw));
        raw_.reset(raw);
    }
    int w() const { return w_; }
    int h() const { return h_; }
    lbm_lattice* raw() const { return raw_.get(); }
    void set_populations(const std::vector<Field>& pops) {
        require(pops.size() == 9, "9 populations");
        Field flat;
        flat.reserve(9 * cells());
        for (const auto& p : pops) {
            require(p.size() == cells(), "population size");
            flat.insert(flat.end(), p.begin(), p.end());
        }
        check(lbm_set_populations(raw(), flat.data()));
    }
    std::vector<Field> populations() const {
        Field flat(9 * cells());
        check(lbm_get_populations(raw(), flat.data()));
        std::vector<Field> out(9);
        for (int i = 0; i < 9; ++i)
            out[i].assign(flat.begin() + i * cells(), flat.begin() + (i + 1) * cells());
        return out;
    }
    void moments(Field& rho, Field& ux, Field& uy) const {
        rho.resize(cells());
        ux.resize(cells());
        uy.resize(cells());
        check(lbm_read_moments(raw(), rho.data(), ux.data(), uy.data(), 0));
    }
    lbm_health health() const {
        lbm_health hs{};
        check(lbm_check(raw(), &hs));
        return hs;
    }
    size_t cells() const { return size_t(w_) * size_t(h_); }

  private:
    struct Del {
        void operator()(lbm_lattice* l) const { lbm_destroy(l); }
    };
    std::unique_ptr<lbm_lattice, Del> raw_;
    int w_, h_;
};

// src/lbm.rs:43-71, evaluated on the GPU.
inline std::vector<Field> compute_equilibrium(const Field& density, const Field& vx,
                                              const Field& vy, int w, int h,
                                              const Discretization& d = {}) {
    require(density.size() == vx.size() && density.size() == vy.size(), "field shapes differ");
    require(density.size() == size_t(w) * size_t(h), "field size");
    Lattice lat(w, h, 1.f);
    check(lbm_set_discretization(lat.raw(), d.delta_x, d.delta_t));
    check(lbm_init_equilibrium(lat.raw(), density.data(), vx.data(), vy.data()));
    return lat.populations();
}

// src/lbm.rs:670-819 on a device lattice.  The collision is BGK or TRT; the
// geometry is w * h booleans (true = solid) or empty.
class State {
  public:
    template <class Collision>
    static State initial(const D2Q9& lattice, std::vector<bool> geometry, const Collision& collision,
                         const Discretization& discretization, int precision = LBM_F32,
                         int flags = LBM_REFERENCE_FLAGS) {
        return State(lattice, std::move(geometry), collision, discretization, precision, flags);
    }

    // State::step (src/lbm.rs:694-714): stream, bounce back, collide, and
    // time += delta_t — fused into one launch per step on the GPU.
    void step(int nsteps = 1) { check(lbm_step(lat_.raw(), nsteps)); }

    Scalar time() const {
        float t = 0.f;
        check(lbm_get_time(lat_.raw(), &t, nullptr));
        return t;
    }
    std::pair<int, int> size() const { return {lat_.w(), lat_.h()}; }
    Scalar delta_x() const { return discretization.delta_x; }
    Scalar delta_t() const { return discretization.delta_t; }
    std::vector<Field> populations() const { return lat_.populations(); }
    Scalar isothermal_speed_of_sound() const { return discretization.isothermal_speed_of_sound(); }

    Field density() const {
        Field r, x, y;
        lat_.moments(r, x, y);
        return r;
    }
    Field pressure() const {
        const Scalar cs = isothermal_speed_of_sound();
        Field p = density();
        for (auto& v : p) v *= cs * cs;
        return p;
    }
    std::pair<Field, Field> velocity() const {
        Field r, x, y;
        lat_.moments(r, x, y);
        return {x, y};
    }
    std::pair<Field, Field> momentum_density() const {
        Field r, x, y;
        lat_.moments(r, x, y);
        for (size_t k = 0; k < r.size(); ++k) {
            x[k] *= r[k];
            y[k] *= r[k];
        }
        return {x, y};
    }
    Field speed() const {
        Field r, x, y;
        lat_.moments(r, x, y);
        for (size_t k = 0; k < r.size(); ++k) r[k] = std::sqrt(x[k] * x[k] + y[k] * y[k]);
        return r;
    }
    std::vector<Field> equilibrium() const {
        Field r, x, y;
        lat_.moments(r, x, y);
        return compute_equilibrium(r, x, y, lat_.w(), lat_.h(), discretization);
    }
    std::vector<Field> non_equilibrium() const {
        auto f = populations();
        const auto eq = equilibrium();
        for (int i = 0; i < 9; ++i)
            for (size_t k = 0; k < f[i].size(); ++k) f[i][k] -= eq[i][k];
        return f;
    }
    // src/lbm.rs:815-818: min over cells of f_eq[0] < 0 (a NaN state counts too)
    bool is_unstable() const {
        const lbm_health hs = lat_.health();
        return hs.min_eq0 < 0.0 || std::isnan(hs.min_eq0) || hs.nonfinite_count > 0;
    }
    const Lattice& device() const { return lat_; }

    // State::geometry, a pub field (src/lbm.rs:670-676) that LBMSim::handle
    // reads and replaces between steps (src/main.rs:77-89): w * h booleans,
    // true = solid, or empty for none.
    const std::vector<bool>& geometry() const { return geometry_; }
    void set_geometry(std::vector<bool> g) {
        require(g.empty() || g.size() == lat_.cells(), "geometry size");
        std::vector<uint8_t> m(g.begin(), g.end());
        check(lbm_set_geometry(lat_.raw(), g.empty() ? nullptr : m.data()));
        geometry_ = std::move(g);
    }

    Discretization discretization;

  private:
    State(const D2Q9& lattice, std::vector<bool> geometry, const BGK& c, const Discretization& d,
          int precision, int flags)
        : discretization(d), lat_(lattice.size().first, lattice.size().second, c.tau, precision, flags) {
        setup(lattice, std::move(geometry));
    }
    State(const D2Q9& lattice, std::vector<bool> geometry, const TRT& c, const Discretization& d,
          int precision, int flags)
        : discretization(d),
          lat_(lattice.size().first, lattice.size().second, c.tau_plus, precision, flags) {
        check(lbm_set_collision(lat_.raw(), LBM_COLLISION_TRT, c.tau_plus, c.tau_minus));
        setup(lattice, std::move(geometry));
    }
    void setup(const D2Q9& lattice, std::vector<bool> geometry) {
        check(lbm_set_discretization(lat_.raw(), discretization.delta_x, discretization.delta_t));
        lat_.set_populations(lattice.pops);
        if (!geometry.empty()) set_geometry(std::move(geometry));
    }
    Lattice lat_;
    std::vector<bool> geometry_;
};

}  // namespace chemsim
