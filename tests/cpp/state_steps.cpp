// Drives the C++ mirror of lbm.rs (include/lbm_state.hpp) the way LBMSim
// drives State<D2Q9> (src/main.rs:128-136): compute_equilibrium of the
// initial fields, State::initial with BGK, n steps, then density / velocity /
// is_unstable / time.  Reads w, h, tau, nsteps and the fields from the input
// file, writes the populations, the moments and is_unstable to the output
// file.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "lbm_state.hpp"

using chemsim::Field;

static void read_into(FILE* fp, void* dst, size_t bytes) {
    if (std::fread(dst, 1, bytes, fp) != bytes) throw std::runtime_error("short input");
}

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s input.bin output.bin\n", argv[0]);
        return 2;
    }
    try {
        FILE* in = std::fopen(argv[1], "rb");
        if (!in) throw std::runtime_error("cannot open input");
        int hdr[4];                                    // w, h, nsteps, has_solid
        float tau = 0.f;
        read_into(in, hdr, sizeof(hdr));
        read_into(in, &tau, sizeof(tau));
        const int w = hdr[0], h = hdr[1], nsteps = hdr[2];
        const size_t n = size_t(w) * h;
        Field rho(n), ux(n), uy(n);
        read_into(in, rho.data(), n * 4);
        read_into(in, ux.data(), n * 4);
        read_into(in, uy.data(), n * 4);
        std::vector<bool> geometry;
        if (hdr[3]) {
            std::vector<uint8_t> g(n);
            read_into(in, g.data(), n);
            geometry.assign(g.begin(), g.end());
        }
        std::fclose(in);

        const chemsim::Discretization disc{1.f, 1.f};
        chemsim::D2Q9 lattice(chemsim::compute_equilibrium(rho, ux, uy, w, h, disc), w, h);
        auto state = chemsim::State::initial(lattice, geometry, chemsim::BGK{tau}, disc);
        for (int s = 0; s < nsteps; ++s) state.step();
        const int unstable = state.is_unstable() ? 1 : 0;
        if (state.time() != float(nsteps) * disc.delta_t) {
            // State::time accumulates delta_t in f32 step by step
            float t = 0.f;
            for (int s = 0; s < nsteps; ++s) t += disc.delta_t;
            if (state.time() != t) throw std::runtime_error("time");
        }
        const auto pops = state.populations();
        const Field density = state.density();
        const auto velocity = state.velocity();
        FILE* out = std::fopen(argv[2], "wb");
        if (!out) throw std::runtime_error("cannot open output");
        for (const auto& p : pops) std::fwrite(p.data(), 4, p.size(), out);
        std::fwrite(density.data(), 4, n, out);
        std::fwrite(velocity.first.data(), 4, n, out);
        std::fwrite(velocity.second.data(), 4, n, out);
        std::fwrite(&unstable, 4, 1, out);
        std::fclose(out);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
