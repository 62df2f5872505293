// lbm_cb8.cuh — the channel-blocked bf16 activation layout of the
// correction network ("CB8"): [image][row + 1][channel block][x + 1][8],
// blocks of 8 channels with a one-pixel zero halo around each image.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>
#include <string.h>

namespace lbmk {

__device__ __forceinline__ uint4 pack8_bf16(const float* v) {
    uint4 r;
    __nv_bfloat162 p0 = __floats2bfloat162_rn(v[0], v[1]);
    __nv_bfloat162 p1 = __floats2bfloat162_rn(v[2], v[3]);
    __nv_bfloat162 p2 = __floats2bfloat162_rn(v[4], v[5]);
    __nv_bfloat162 p3 = __floats2bfloat162_rn(v[6], v[7]);
    memcpy(&r.x, &p0, 4);
    memcpy(&r.y, &p1, 4);
    memcpy(&r.z, &p2, 4);
    memcpy(&r.w, &p3, 4);
    return r;
}
__device__ __forceinline__ void unpack8_bf16(uint4 r, float* v) {
    __nv_bfloat162 p[4];
    memcpy(&p[0], &r.x, 4);
    memcpy(&p[1], &r.y, 4);
    memcpy(&p[2], &r.z, 4);
    memcpy(&p[3], &r.w, 4);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float2 f = __bfloat1622float2(p[k]);
        v[2 * k] = f.x;
        v[2 * k + 1] = f.y;
    }
}

// CB8 offset (in 8-channel chunks) of pixel (x, y) of block cb.
__host__ __device__ __forceinline__ int64_t cb8_chunk(int b, int y, int cb, int x, int H, int W,
                                                      int CB) {
    return ((int64_t(b) * (H + 2) + (y + 1)) * CB + cb) * (W + 2) + (x + 1);
}

}  // namespace lbmk
