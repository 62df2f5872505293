// lbm_coarse.cu — the lattice side of the learned coarse-grid correction:
// restriction of a fine lattice onto a coarser one, the correction network's
// input features, the application of its population correction and the
// training target (the population change that moves the coarse velocity
// onto the restricted fine one).
// No reference counterpart.
#include <string>

#include "lbm_cb8.cuh"
#include "lbm_handle.cuh"

using namespace lbmk;

namespace {

// Network input from a lattice's moments, image b of an NCHW f32 tensor
// (batch, 4, H, W): (rho - 1) * s_rho, ux * s_u, uy * s_u on fluid cells,
// zero on solid ones, and the solid flag.
__global__ void features_kernel(const float* __restrict__ rho, const float* __restrict__ ux,
                                const float* __restrict__ uy, int pitch,
                                const uint8_t* __restrict__ solid, int mpitch, int H, int W,
                                float s_rho, float s_u, int b, float* __restrict__ out) {
    const int64_t n = int64_t(H) * W;
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n;
         e += int64_t(gridDim.x) * blockDim.x) {
        const int y = int(e / W), x = int(e % W);
        const int64_t o = int64_t(y) * pitch + x;
        const bool s = solid != nullptr && solid[int64_t(y) * mpitch + x];
        float* img = out + int64_t(b) * 4 * n;
        img[e] = s ? 0.f : (rho[o] - 1.f) * s_rho;
        img[n + e] = s ? 0.f : ux[o] * s_u;
        img[2 * n + e] = s ? 0.f : uy[o] * s_u;
        img[3 * n + e] = s ? 1.f : 0.f;
    }
}

// Raw density and velocity j / rho of a stored f32 cell.
__device__ __forceinline__ void raw_moments(const float (&f)[9], float& rho, float& ux, float& uy) {
    rho = ((f[0] + f[1]) + (f[2] + f[3])) + ((f[4] + f[5]) + (f[6] + f[7])) + f[8];
    const float jx = (f[1] - f[3]) + (f[5] - f[6]) + (f[8] - f[7]);
    const float jy = (f[2] - f[4]) + (f[5] + f[6]) - (f[7] + f[8]);
    ux = jx / rho;
    uy = jy / rho;
}

// Population correction of the fluid cells of an f32 lattice: d_i = scale *
// corr[b][i] (clamped to +-max_abs when max_abs > 0), applied as
// f_i += d_i - w_i sum_j d_j so that the cell's mass does not change.
__global__ void apply_correction_kernel(float* __restrict__ f, int64_t plane, int pitch,
                                        const uint8_t* __restrict__ solid, int mpitch, int H, int W,
                                        const float* __restrict__ corr, int b, float scale,
                                        float max_abs) {
    const int64_t n = int64_t(H) * W;
    const float w[9] = {16.f / 36.f, 4.f / 36.f, 4.f / 36.f, 4.f / 36.f, 4.f / 36.f,
                        1.f / 36.f, 1.f / 36.f, 1.f / 36.f, 1.f / 36.f};
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n;
         e += int64_t(gridDim.x) * blockDim.x) {
        const int y = int(e / W), x = int(e % W);
        if (solid != nullptr && solid[int64_t(y) * mpitch + x]) continue;
        const int64_t o = int64_t(y) * pitch + x;
        float d[9], sum = 0.f;
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            d[i] = scale * corr[(int64_t(b) * 9 + i) * n + e];
            if (max_abs > 0.f) d[i] = fminf(fmaxf(d[i], -max_abs), max_abs);
            sum += d[i];
        }
#pragma unroll
        for (int i = 0; i < 9; ++i) f[i * plane + o] += d[i] - w[i] * sum;
    }
}

// target[b][i] = (f_eq_i(rho_cur, u_ref) - f_eq_i(rho_cur, u_cur)) / scale
// with u = j / rho of the stored states (ref holds equilibria, written by the
// restriction); zero on solid cells.  The target moves cur's velocity onto
// ref's and changes neither its density nor its non-equilibrium part.
__global__ void velocity_shift_kernel(const float* __restrict__ ref, const float* __restrict__ cur,
                                      int64_t plane, int pitch, const uint8_t* __restrict__ solid,
                                      int mpitch, int H, int W, float inv_scale, int b,
                                      float* __restrict__ target, Consts<float> c) {
    const int64_t n = int64_t(H) * W;
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n;
         e += int64_t(gridDim.x) * blockDim.x) {
        const int y = int(e / W), x = int(e % W);
        const int64_t o = int64_t(y) * pitch + x;
        float* t = target + int64_t(b) * 9 * n + e;
        if (solid != nullptr && solid[int64_t(y) * mpitch + x]) {
#pragma unroll
            for (int i = 0; i < 9; ++i) t[i * n] = 0.f;
            continue;
        }
        float fr[9], fc[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            fr[i] = ref[i * plane + o];
            fc[i] = cur[i * plane + o];
        }
        float rr, rx, ry, rc, cx, cy;
        raw_moments(fr, rr, rx, ry);
        raw_moments(fc, rc, cx, cy);
        float e0[9], e1[9];
        equilibrium_strict<float>(c, rc, cx, cy, e0);
        equilibrium_strict<float>(c, rc, rx, ry, e1);
#pragma unroll
        for (int i = 0; i < 9; ++i) t[i * n] = (e1[i] - e0[i]) * inv_scale;
    }
}

// Coarse populations = f_eq of block-averaged fine moments: rho_c = mean rho
// over the fluid fine cells of the block (1 if none), u_c = sum(rho u) /
// sum(rho), shifted by +F_c/2 / rho_c so that the coarse lattice reads back
// u_c under its own forcing convention.
__global__ void restrict_kernel(const float* __restrict__ rho, const float* __restrict__ ux,
                                const float* __restrict__ uy, int fpitch,
                                const uint8_t* __restrict__ fsolid, int fmpitch, int factor,
                                float* __restrict__ cf, int64_t cplane, int cpitch, int Hc, int Wc,
                                float hfx, float hfy, Consts<float> c) {
    const int64_t n = int64_t(Hc) * Wc;
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n;
         e += int64_t(gridDim.x) * blockDim.x) {
        const int Y = int(e / Wc), X = int(e % Wc);
        double sr = 0.0, sjx = 0.0, sjy = 0.0;
        int cnt = 0;
        for (int dy = 0; dy < factor; ++dy)
            for (int dx = 0; dx < factor; ++dx) {
                const int y = Y * factor + dy, x = X * factor + dx;
                if (fsolid != nullptr && fsolid[int64_t(y) * fmpitch + x]) continue;
                const int64_t o = int64_t(y) * fpitch + x;
                sr += rho[o];
                sjx += double(rho[o]) * ux[o];
                sjy += double(rho[o]) * uy[o];
                ++cnt;
            }
        float r = 1.f, vx = 0.f, vy = 0.f;
        if (cnt > 0 && sr > 0.0) {
            r = float(sr / cnt);
            vx = float(sjx / sr) + hfx / r;
            vy = float(sjy / sr) + hfy / r;
        }
        float feq[9];
        equilibrium_strict<float>(c, r, vx, vy, feq);
        const int64_t o = int64_t(Y) * cpitch + X;
#pragma unroll
        for (int i = 0; i < 9; ++i) cf[i * cplane + o] = feq[i];
    }
}

int grid_of(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    if (g > 65535 * 4) g = 65535 * 4;
    return int(g < 1 ? 1 : g);
}

int kfail(int code, const std::string& msg) { return lattice_fail(code, msg); }

#define CO_CUDA(expr)                                                                      \
    do {                                                                                   \
        cudaError_t e__ = (expr);                                                          \
        if (e__ != cudaSuccess) {                                                          \
            (void)cudaGetLastError();                                                      \
            return kfail(LBM_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e__)); \
        }                                                                                  \
    } while (0)

bool f32_lattice(const lbm_lattice* L) { return L && L->precision == LBM_F32; }

}  // namespace

extern "C" {

int lbm_restrict(lbm_lattice* fine, lbm_lattice* coarse, int factor) {
    if (!fine || !coarse) return kfail(LBM_ERR_INVALID_ARGUMENT, "null lattice");
    if (factor < 1 || fine->w != coarse->w * factor || fine->h != coarse->h * factor)
        return kfail(LBM_ERR_INVALID_ARGUMENT, "coarse sides must be the fine sides / factor");
    if (!f32_lattice(fine) || !f32_lattice(coarse))
        return kfail(LBM_ERR_NOT_SUPPORTED, "restriction needs f32 lattices");
    if (int rc = lattice_refresh_moments(fine)) return rc;
    CO_CUDA(cudaStreamSynchronize(fine->stream));
    const Consts<float> c = lattice_args<float>(coarse, coarse->cur, false).c;
    const int64_t n = int64_t(coarse->w) * coarse->h;
    restrict_kernel<<<grid_of(n, 256), 256, 0, coarse->stream>>>(
        fine->mom[0], fine->mom[1], fine->mom[2], fine->pitch,
        fine->has_solid ? fine->solid : nullptr, fine->mpitch, factor,
        static_cast<float*>(coarse->buf[coarse->cur]), coarse->plane, coarse->pitch, coarse->h,
        coarse->w, 0.5f * coarse->fx, 0.5f * coarse->fy, c);
    CO_CUDA(cudaGetLastError());
    CO_CUDA(cudaStreamSynchronize(coarse->stream));
    coarse->mom_valid = false;
    return LBM_OK;
}

int lbm_coarse_features(lbm_lattice* lat, float s_rho, float s_u, int image, float* in) {
    if (!lat || !in || image < 0) return kfail(LBM_ERR_INVALID_ARGUMENT, "bad argument");
    if (int rc = lattice_refresh_moments(lat)) return rc;
    features_kernel<<<grid_of(int64_t(lat->w) * lat->h, 256), 256, 0, lat->stream>>>(
        lat->mom[0], lat->mom[1], lat->mom[2], lat->pitch, lat->has_solid ? lat->solid : nullptr,
        lat->mpitch, lat->h, lat->w, s_rho, s_u, image, in);
    CO_CUDA(cudaGetLastError());
    return LBM_OK;
}

int lbm_coarse_apply(lbm_lattice* lat, const float* corr, int image, float scale, float max_abs) {
    if (!f32_lattice(lat) || !corr || image < 0 || !(max_abs >= 0.f))
        return kfail(LBM_ERR_INVALID_ARGUMENT, "need an f32 lattice, a correction and max_abs >= 0");
    apply_correction_kernel<<<grid_of(int64_t(lat->w) * lat->h, 256), 256, 0, lat->stream>>>(
        static_cast<float*>(lat->buf[lat->cur]), lat->plane, lat->pitch,
        lat->has_solid ? lat->solid : nullptr, lat->mpitch, lat->h, lat->w, corr, image, scale,
        max_abs);
    CO_CUDA(cudaGetLastError());
    lat->mom_valid = false;
    return LBM_OK;
}

int lbm_coarse_target(lbm_lattice* ref, lbm_lattice* cur, float scale, int image, float* target) {
    if (!f32_lattice(ref) || !f32_lattice(cur) || !target || image < 0 || !(scale > 0.f))
        return kfail(LBM_ERR_INVALID_ARGUMENT, "need two f32 lattices, a target and scale > 0");
    if (ref->w != cur->w || ref->h != cur->h) return kfail(LBM_ERR_INVALID_ARGUMENT, "size mismatch");
    CO_CUDA(cudaStreamSynchronize(ref->stream));
    velocity_shift_kernel<<<grid_of(int64_t(cur->w) * cur->h, 256), 256, 0, cur->stream>>>(
        static_cast<const float*>(ref->buf[ref->cur]), static_cast<const float*>(cur->buf[cur->cur]),
        cur->plane, cur->pitch, cur->has_solid ? cur->solid : nullptr, cur->mpitch, cur->h, cur->w,
        1.f / scale, image, target, lattice_args<float>(cur, cur->cur, false).c);
    CO_CUDA(cudaGetLastError());
    return LBM_OK;
}

}  // extern "C"
