// lbm_step.cuh — the fused D2Q9 step kernel (sm_103a).
//
// One launch = one time step of State::step (taktoa/chemsim
// src/lbm.rs:694-714): pull streaming (stream, :716-729), bounce-back
// (:741-751, or its half-way variant), moments, equilibrium
// (compute_equilibrium, :43-71) and relaxation (BGK :350-364 / TRT
// :399-446), fused so each population is read once and written once.
//
// Layout: 9 structure-of-arrays planes, rows of `pitch` elements (a multiple
// of 128 bytes), x contiguous.  A warp owns 32*V consecutive cells of one row;
// each lane loads V cells of a plane with one aligned vector load (16 bytes
// for f32 V=4, f64 V=2, 16-bit V=8).  The +-1 column shifts of the pull are
// realigned in registers with warp shuffles, so every global load is an
// aligned, coalesced vector; only the two lanes at a warp's ends fetch one
// extra scalar (an L1/L2 hit).  Row shifts are plain row offsets.
#pragma once

#include "lbm_common.cuh"

namespace lbmk {

constexpr unsigned kFull = 0xffffffffu;

template <class S, int V>
struct VecIO {
    static constexpr int BYTES = int(sizeof(S)) * V;
    static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16 || BYTES == 32, "vector width");
    __device__ __forceinline__ static void load(const S* p, S (&out)[V]) {
        if constexpr (BYTES == 32) {
            const uint4* q = reinterpret_cast<const uint4*>(p);
            uint4 r[2] = {__ldg(q), __ldg(q + 1)};
            memcpy(out, r, 32);
        } else if constexpr (BYTES == 16) {
            uint4 r = __ldg(reinterpret_cast<const uint4*>(p));
            memcpy(out, &r, 16);
        } else if constexpr (BYTES == 8) {
            uint2 r = __ldg(reinterpret_cast<const uint2*>(p));
            memcpy(out, &r, 8);
        } else {
            unsigned r = __ldg(reinterpret_cast<const unsigned*>(p));
            memcpy(out, &r, 4);
        }
    }
    __device__ __forceinline__ static void store(S* p, const S (&v)[V]) {
        if constexpr (BYTES == 32) {
            uint4 r[2];
            memcpy(r, v, 32);
            reinterpret_cast<uint4*>(p)[0] = r[0];
            reinterpret_cast<uint4*>(p)[1] = r[1];
        } else if constexpr (BYTES == 16) {
            uint4 r;
            memcpy(&r, v, 16);
            *reinterpret_cast<uint4*>(p) = r;
        } else if constexpr (BYTES == 8) {
            uint2 r;
            memcpy(&r, v, 8);
            *reinterpret_cast<uint2*>(p) = r;
        } else {
            unsigned r;
            memcpy(&r, v, 4);
            *reinterpret_cast<unsigned*>(p) = r;
        }
    }
};

template <int V>
__device__ __forceinline__ uint32_t load_mask_core(const uint8_t* p) {
    uint32_t bits = 0;
    if constexpr (V == 8) {
        const uint2 r = __ldg(reinterpret_cast<const uint2*>(p));
#pragma unroll
        for (int k = 0; k < 4; ++k) bits |= (((r.x >> (8 * k)) & 0xffu) != 0u) << k;
#pragma unroll
        for (int k = 0; k < 4; ++k) bits |= (((r.y >> (8 * k)) & 0xffu) != 0u) << (k + 4);
    } else if constexpr (V == 4) {
        const unsigned r = __ldg(reinterpret_cast<const unsigned*>(p));
#pragma unroll
        for (int k = 0; k < 4; ++k) bits |= (((r >> (8 * k)) & 0xffu) != 0u) << k;
    } else if constexpr (V == 2) {
        const unsigned short r = __ldg(reinterpret_cast<const unsigned short*>(p));
        bits = ((r & 0xffu) != 0u) | ((((r >> 8) & 0xffu) != 0u) << 1);
    } else {
        bits = __ldg(p) != 0;
    }
    return bits;
}

// Solid bit of column col of a mask row, with the x-axis rule for columns
// outside [0, w): wrapped when periodic, 0 otherwise (the axis rule decides).
__device__ __forceinline__ uint32_t mask_at(const uint8_t* row, int col, int w, bool xper) {
    if (col >= 0 && col < w) return __ldg(row + col) != 0;
    if (xper) {
        int c = col % w;
        if (c < 0) c += w;
        return __ldg(row + c) != 0;
    }
    return 0;
}

// Bits j = 0..V+1 <-> solid(column x0 - 1 + j) of one mask row.
template <int V>
__device__ __forceinline__ uint32_t mask_row_bits(const uint8_t* row, int x0, int xl,
                                                  int w, int lane, bool xper) {
    uint32_t core = load_mask_core<V>(row + xl);
    uint32_t left = __shfl_up_sync(kFull, (core >> (V - 1)) & 1u, 1);
    uint32_t right = __shfl_down_sync(kFull, core & 1u, 1);
    if (lane == 0 || x0 == 0) left = mask_at(row, x0 - 1, w, xper);
    if (lane == 31 || x0 + V >= w) {
        right = mask_at(row, x0 + V, w, xper);
#pragma unroll
        for (int k = 0; k < V; ++k)
            if (x0 + k >= w) core = (core & ~(1u << k)) | (mask_at(row, x0 + k, w, xper) << k);
    }
    return left | (core << 1) | (right << (V + 1));
}

// The collision of one cell: f (pre-collision, post-streaming) -> out.
template <bool FAST, class CT>
__device__ __forceinline__ void collide_cell(const Consts<CT>& c, const CT (&f)[9], CT (&out)[9]) {
    using A = Ar<FAST>;
    // density (src/lbm.rs:117-121) and momentum_density (:123-131); the terms
    // f_i * 0 and the +-1 products are exact, so the nonzero terms are summed
    // in the reference's order.
    CT rho = A::add(CT(0), f[0]);
#pragma unroll
    for (int i = 1; i < 9; ++i) rho = A::add(rho, f[i]);
    CT mx = A::sub(f[1], f[3]);
    mx = A::add(mx, f[5]);
    mx = A::sub(mx, f[6]);
    mx = A::sub(mx, f[7]);
    mx = A::add(mx, f[8]);
    CT my = A::sub(f[2], f[4]);
    my = A::add(my, f[5]);
    my = A::add(my, f[6]);
    my = A::sub(my, f[7]);
    my = A::sub(my, f[8]);
    if (c.force) { mx = A::add(mx, c.hfx); my = A::add(my, c.hfy); }
    const CT inv = A::rcp(rho);                 // Matrix::recip (src/matrix.rs:133-136)
    const CT ux = A::mul(inv, mx);
    const CT uy = A::mul(inv, my);
    const CT v2k3 = A::mul(A::add(A::mul(ux, ux), A::mul(uy, uy)), c.k3);
    // c_i . u for each direction (exact negations of the reference's products).
    CT vc[9];
    vc[0] = CT(0);
    vc[1] = ux;
    vc[2] = uy;
    vc[3] = -ux;
    vc[4] = -uy;
    vc[5] = A::add(ux, uy);
    vc[6] = A::sub(uy, ux);
    vc[7] = -vc[5];
    vc[8] = A::sub(ux, uy);
    const CT rw0 = A::mul(rho, c.wt[0]);
    const CT rw1 = A::mul(rho, c.wt[1]);
    const CT rw5 = A::mul(rho, c.wt[5]);
    CT feq[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const CT rw = i == 0 ? rw0 : (i < 5 ? rw1 : rw5);
        CT s;
        if constexpr (FAST) {
            s = fma(vc[i], c.k1, CT(1));
            s = fma(vc[i] * vc[i], c.k2, s);
            s = s + v2k3;
        } else {
            s = A::add(CT(1), A::mul(vc[i], c.k1));
            s = A::add(s, A::mul(A::mul(vc[i], vc[i]), c.k2));
            s = A::add(s, v2k3);
        }
        feq[i] = A::mul(rw, s);
    }
    if (c.collision == LBM_COLLISION_TRT) {
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const int o = OPP(i);
            const CT fsw = f[o];
            // swap_equilibrium fills entries 1..8 from the populations
            // (src/lbm.rs:311-322); kept as written.
            const CT eqsw = (i == 0) ? feq[0] : f[o];
            const CT fp = A::add(f[i], fsw);
            const CT fm = A::sub(f[i], fsw);
            const CT ep = A::add(feq[i], eqsw);
            const CT em = A::sub(feq[i], eqsw);
            const CT om = A::mul(A::add(A::mul(A::sub(fp, ep), c.omega_p),
                                        A::mul(A::sub(fm, em), c.omega_m)),
                                 c.trt_scale);
            out[i] = A::add(f[i], om);
        }
    } else {
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            if constexpr (FAST) out[i] = fma(f[i] - feq[i], c.bgk_factor, f[i]);
            else out[i] = A::add(f[i], A::mul(A::sub(f[i], feq[i]), c.bgk_factor));
        }
    }
    if (c.force) {
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const CT cx = CT(CX(i)), cy = CT(CY(i));
            const CT vci = A::add(A::mul(ux, cx), A::mul(uy, cy));
            const CT t1 = A::mul(A::add(A::mul(A::sub(cx, ux), c.fx),
                                        A::mul(A::sub(cy, uy), c.fy)), c.k1);
            const CT t2 = A::mul(A::mul(vci, A::add(A::mul(cx, c.fx), A::mul(cy, c.fy))),
                                 c.inv_cs4);
            const CT wg = A::mul(c.guo, c.wt[i]);
            out[i] = A::add(out[i], A::mul(wg, A::add(t1, t2)));
        }
    }
}

// Moments of a stored cell state (Lattice::density / velocity, src/lbm.rs:
// 117-149), with u = (j - F/2)/rho when a body force is set.
template <bool FAST, class CT>
__device__ __forceinline__ void cell_moments(const Consts<CT>& c, const CT (&f)[9],
                                             CT& rho, CT& ux, CT& uy) {
    using A = Ar<FAST>;
    rho = A::add(CT(0), f[0]);
#pragma unroll
    for (int i = 1; i < 9; ++i) rho = A::add(rho, f[i]);
    CT mx = A::sub(f[1], f[3]);
    mx = A::add(mx, f[5]);
    mx = A::sub(mx, f[6]);
    mx = A::sub(mx, f[7]);
    mx = A::add(mx, f[8]);
    CT my = A::sub(f[2], f[4]);
    my = A::add(my, f[5]);
    my = A::add(my, f[6]);
    my = A::sub(my, f[7]);
    my = A::sub(my, f[8]);
    if (c.force) { mx = A::sub(mx, c.hfx); my = A::sub(my, c.hfy); }
    const CT inv = A::rcp(rho);
    ux = A::mul(inv, mx);
    uy = A::mul(inv, my);
}

template <class S, int V, int FRAME, bool FAST>
__global__ void __launch_bounds__(256)
lbm_step_kernel(const StepArgs<typename Store<S>::CT> a) {
    using CT = typename Store<S>::CT;
    using ST = Store<S>;
    using IO = VecIO<S, V>;
    constexpr uint32_t FULL = (1u << V) - 1u;

    const int lane = threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (y >= a.h) return;                       // warp-uniform
    const int w = a.w, h = a.h;
    const int x0 = (blockIdx.x * 32 + lane) * V;
    const bool active = x0 < w;
    const int xl = active ? x0 : 0;            // idle lanes read a valid chunk
    const S* __restrict__ src = static_cast<const S*>(a.src);
    S* __restrict__ dst = static_cast<S*>(a.dst);
    const int64_t P = a.pitch, PL = a.plane;
    const int xm = a.flags & 3, ym = (a.flags >> 2) & 3;
    const bool halfway = (a.flags & LBM_SOLID_HALFWAY) != 0;
    const bool has_solid = a.solid != nullptr;
    const bool xper = xm == 1;

    // Solid bits of rows y-1, y, y+1 (index 1 - drow of a direction).
    uint32_t mrow[3] = {0u, 0u, 0u};
    if (has_solid) {
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            int row = y - 1 + r;
            bool ok = true;
            if (row < 0 || row >= h) {
                if (ym == 1) row = row < 0 ? row + h : row - h;
                else ok = false;
            }
            if (ok)   // warp-uniform
                mrow[r] = mask_row_bits<V>(a.solid + int64_t(row) * a.mpitch, x0, xl, w, lane, xper);
        }
    }

    CT f[9][V];
    uint32_t bnc[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const int dc = DCOL(FRAME, i), dr = DROW(FRAME, i);
        int sr = y - dr;
        int rowcls = 0;                          // 0 cells, 1 zero, 2 bounce
        if (sr < 0 || sr >= h) {
            if (ym == 1) sr = sr < 0 ? sr + h : sr - h;
            else rowcls = (ym == 2) ? 2 : 1;
        }
        const S* plane = src + i * PL;
        const S* prow = plane + int64_t(rowcls == 0 ? sr : 0) * P;
        const CT wi = a.c.wt[i];
        CT v[V];
        {
            S raw[V];
            IO::load(prow + xl, raw);
#pragma unroll
            for (int k = 0; k < V; ++k) v[k] = ST::dec(raw[k], wi, a.c.dinv);
        }
        uint32_t xz = 0u, xb = 0u;
        if (dc == 1) {
            const CT left = __shfl_up_sync(kFull, v[V - 1], 1);
#pragma unroll
            for (int k = V - 1; k > 0; --k) v[k] = v[k - 1];
            v[0] = left;
            if (lane == 0 || x0 == 0) {
                int sx = x0 - 1;
                if (sx >= 0) v[0] = ST::dec(__ldg(prow + sx), wi, a.c.dinv);
                else if (xper) v[0] = ST::dec(__ldg(prow + sx + w), wi, a.c.dinv);
                else if (xm == 2) xb |= 1u;
                else xz |= 1u;
            }
        } else if (dc == -1) {
            const CT right = __shfl_down_sync(kFull, v[0], 1);
#pragma unroll
            for (int k = 0; k < V - 1; ++k) v[k] = v[k + 1];
            v[V - 1] = right;
            if (lane == 31 || x0 + V >= w) {
#pragma unroll
                for (int k = 0; k < V; ++k) {
                    const int sx = x0 + k + 1;
                    if (sx >= w) {
                        if (xper) v[k] = ST::dec(__ldg(prow + (sx % w)), wi, a.c.dinv);
                        else if (xm == 2) xb |= 1u << k;
                        else xz |= 1u << k;
                    } else if (k == V - 1) {
                        v[k] = ST::dec(__ldg(prow + sx), wi, a.c.dinv);
                    }
                }
            }
        }
        uint32_t b = (rowcls == 2) ? FULL : xb;
        const uint32_t z = (rowcls == 1 ? FULL : xz) & ~b;
        if (has_solid && halfway) b |= (mrow[1 - dr] >> (1 - dc)) & FULL;
#pragma unroll
        for (int k = 0; k < V; ++k) f[i][k] = ((z >> k) & 1u) ? CT(0) : v[k];
        bnc[i] = b;
    }

    // Bounce-back links: the cell's own post-collision opposite population.
#pragma unroll
    for (int i = 1; i < 9; ++i) {
        if (bnc[i]) {
            S raw[V];
            IO::load(src + OPP(i) * PL + int64_t(y) * P + xl, raw);
#pragma unroll
            for (int k = 0; k < V; ++k)
                if ((bnc[i] >> k) & 1u) f[i][k] = ST::dec(raw[k], a.c.wt[OPP(i)], a.c.dinv);
        }
    }

    const uint32_t own_solid = has_solid ? ((mrow[1] >> 1) & FULL) : 0u;
    if (own_solid && !halfway) {
        // bounce_back (src/lbm.rs:741-751): solid nodes take swapped populations.
#pragma unroll
        for (int k = 0; k < V; ++k) {
            if ((own_solid >> k) & 1u) {
                CT t;
                t = f[1][k]; f[1][k] = f[3][k]; f[3][k] = t;
                t = f[2][k]; f[2][k] = f[4][k]; f[4][k] = t;
                t = f[5][k]; f[5][k] = f[7][k]; f[7][k] = t;
                t = f[6][k]; f[6][k] = f[8][k]; f[8][k] = t;
            }
        }
    }

    // Collide and write.
    CT out[9][V];
#pragma unroll
    for (int k = 0; k < V; ++k) {
        CT g[9], o[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) g[i] = f[i][k];
        collide_cell<FAST>(a.c, g, o);
#pragma unroll
        for (int i = 0; i < 9; ++i) out[i][k] = o[i];
    }
    S enc[9][V];
#pragma unroll
    for (int i = 0; i < 9; ++i)
#pragma unroll
        for (int k = 0; k < V; ++k) enc[i][k] = ST::enc(out[i][k], a.c.wt[i], a.c.dscale);

    if (own_solid && halfway) {
        // Half-way mode: solid nodes keep their populations.
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            S raw[V];
            IO::load(src + i * PL + int64_t(y) * P + xl, raw);
#pragma unroll
            for (int k = 0; k < V; ++k)
                if ((own_solid >> k) & 1u) enc[i][k] = raw[k];
        }
    }

    if (!active) return;
    const int64_t base = int64_t(y) * P + x0;
    if (x0 + V <= w) {
#pragma unroll
        for (int i = 0; i < 9; ++i) IO::store(dst + i * PL + base, enc[i]);
    } else {
#pragma unroll
        for (int i = 0; i < 9; ++i)
#pragma unroll
            for (int k = 0; k < V; ++k)
                if (x0 + k < w) dst[i * PL + base + k] = enc[i][k];
    }

    if (a.mom_rho != nullptr) {
#pragma unroll
        for (int k = 0; k < V; ++k) {
            if (x0 + k >= w) break;
            CT g[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) g[i] = ST::dec(enc[i][k], a.c.wt[i], a.c.dinv);
            CT r, ux, uy;
            cell_moments<FAST>(a.c, g, r, ux, uy);
            a.mom_rho[base + k] = float(r);
            a.mom_ux[base + k] = float(ux);
            a.mom_uy[base + k] = float(uy);
        }
    }
}

template <class S, int V>
cudaError_t launch_step_v(const StepArgs<typename Store<S>::CT>& a, int frame, bool fast,
                          int rows, cudaStream_t stream) {
    const dim3 block(32, rows);
    const dim3 grid((a.w + 32 * V - 1) / (32 * V), (a.h + rows - 1) / rows);
    if (frame) {
        if (fast) lbm_step_kernel<S, V, 1, true><<<grid, block, 0, stream>>>(a);
        else lbm_step_kernel<S, V, 1, false><<<grid, block, 0, stream>>>(a);
    } else {
        if (fast) lbm_step_kernel<S, V, 0, true><<<grid, block, 0, stream>>>(a);
        else lbm_step_kernel<S, V, 0, false><<<grid, block, 0, stream>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace lbmk
