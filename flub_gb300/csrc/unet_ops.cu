// U-Net pieces around the tcgen05 convolution (unet_conv.cu): input assembly,
// 2x pooling / upsampling and their gradients, ReLU gradient, the 1x1x1 output
// head, the masked MSE loss, the convolution weight gradient, and Adam.
//
// No reference counterpart: the learned warm start is an addition to the
// projection (the reference always starts CG from x = 0).  Activations are
// channels-last BF16 [B][X][Y][Z][C]; parameters, gradients and optimiser
// state are FP32.
#include <cuda_bf16.h>

#include "common.cuh"

namespace flub {

#define GRID_LOOP(i, n) for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }

// Per-sample 1 / RMS of the right-hand side over fluid cells (1 if none), in
// two deterministic passes: kRmsBlocks blocks per sample write (sum, count)
// partials, one block per sample combines them in index order.
constexpr int kRmsBlocks = 152;

__global__ void __launch_bounds__(256) k_unet_rms_part(const float *__restrict__ div, const int32_t *__restrict__ tag,
                                                       int64_t ncell, double *__restrict__ work) {
    __shared__ double red[32], cnt_red[32];
    const int b = blockIdx.y;
    double s = 0.0, c = 0.0;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < ncell; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = b * ncell + q;
        if (tag[v] == 1) {
            const double d = div[v];
            s += d * d;
            c += 1.0;
        }
    }
    s = block_sum(s, red);
    c = block_sum(c, cnt_red);
    if (threadIdx.x == 0) {
        work[2 * ((int64_t)b * gridDim.x + blockIdx.x)] = s;
        work[2 * ((int64_t)b * gridDim.x + blockIdx.x) + 1] = c;
    }
}

__global__ void __launch_bounds__(256) k_unet_rms_final(const double *__restrict__ work, int parts,
                                                        float *__restrict__ inv_scale) {
    __shared__ double red[32], cnt_red[32];
    const int b = blockIdx.x;
    double s = 0.0, c = 0.0;
    for (int q = threadIdx.x; q < parts; q += blockDim.x) {
        s += work[2 * ((int64_t)b * parts + q)];
        c += work[2 * ((int64_t)b * parts + q) + 1];
    }
    s = block_sum(s, red);
    c = block_sum(c, cnt_red);
    if (threadIdx.x == 0) inv_scale[b] = (c > 0.0 && s > 0.0) ? (float)(1.0 / sqrt(s / c)) : 1.0f;
}

// Network input, 16 channels: div / rms, fluid mask, solid mask, 13 zeros.
__global__ void __launch_bounds__(256) k_unet_input(const float *__restrict__ div, const int32_t *__restrict__ tag,
                                                    const float *__restrict__ inv_scale, int64_t ncell, int64_t n,
                                                    __nv_bfloat16 *__restrict__ out) {
    GRID_LOOP(v, n) {
        const int b = (int)(v / ncell);
        const int t = tag[v];
        __align__(16) __nv_bfloat16 ch[16];
#pragma unroll
        for (int c = 0; c < 16; c++) ch[c] = __float2bfloat16_rn(0.0f);
        ch[0] = __float2bfloat16_rn(t == 1 ? div[v] * inv_scale[b] : 0.0f);
        ch[1] = __float2bfloat16_rn(t == 1 ? 1.0f : 0.0f);
        ch[2] = __float2bfloat16_rn(t == 2 ? 1.0f : 0.0f);
        uint4 *dst = reinterpret_cast<uint4 *>(out + v * 16);
        dst[0] = reinterpret_cast<const uint4 *>(ch)[0];
        dst[1] = reinterpret_cast<const uint4 *>(ch)[1];
    }
}

// 2x average pool (fine -> coarse), C channels.
__global__ void __launch_bounds__(256) k_pool2(const __nv_bfloat16 *__restrict__ x, __nv_bfloat16 *__restrict__ y,
                                               int B, int NX, int NY, int NZ, int C) {
    const int cx = NX / 2, cy = NY / 2, cz = NZ / 2;
    const int64_t n = (int64_t)B * cx * cy * cz * C;
    GRID_LOOP(q, n) {
        const int c = (int)(q % C);
        int64_t v = q / C;
        const int k = (int)(v % cz); v /= cz;
        const int j = (int)(v % cy); v /= cy;
        const int i = (int)(v % cx);
        const int b = (int)(v / cx);
        float s = 0.0f;
        for (int d = 0; d < 8; d++) {
            const int64_t f = ((((int64_t)b * NX + 2 * i + (d >> 2)) * NY + 2 * j + ((d >> 1) & 1)) * NZ + 2 * k + (d & 1));
            s += bf(x[f * C + c]);
        }
        y[q] = __float2bfloat16_rn(s * 0.125f);
    }
}

// The same pool for C % 8 == 0: thread t of coarse row (b, i, j) averages
// channels 8 c8 .. 8 c8 + 7 of coarse voxel k = t / (C / 8) from its 8 fine
// voxels (16-byte loads), summing them in k_pool2's order.
// Grid: (ceil((NZ / 2) * (C / 8) / 128), NY / 2, B * (NX / 2)), 128 threads.
__global__ void __launch_bounds__(128) k_pool2_v8(const uint4 *__restrict__ x, uint4 *__restrict__ y, int NX, int NY,
                                                  int NZ, int C8) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int cx = NX >> 1, cy = NY >> 1, cz = NZ >> 1;
    if (t >= cz * C8) return;
    const int k = t / C8, c8 = t - k * C8;
    const int j = blockIdx.y, bi = blockIdx.z;
    const int b = bi / cx, i = bi - b * cx;
    float s[8];
#pragma unroll
    for (int m = 0; m < 8; m++) s[m] = 0.0f;
#pragma unroll
    for (int d = 0; d < 8; d++) {
        const int64_t f = (((int64_t)b * NX + 2 * i + (d >> 2)) * NY + 2 * j + ((d >> 1) & 1)) * NZ + 2 * k + (d & 1);
        const uint4 u = __ldg(x + f * C8 + c8);
        const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float2 p = __bfloat1622float2(h[q]);
            s[2 * q] += p.x;
            s[2 * q + 1] += p.y;
        }
    }
    uint4 o;
    __nv_bfloat162 *oh = reinterpret_cast<__nv_bfloat162 *>(&o);
#pragma unroll
    for (int q = 0; q < 4; q++) oh[q] = __floats2bfloat162_rn(s[2 * q] * 0.125f, s[2 * q + 1] * 0.125f);
    y[(((int64_t)bi * cy + j) * cz + k) * C8 + c8] = o;
}

// Gradient of the pool: dx (+)= dy / 8.
__global__ void __launch_bounds__(256) k_pool2_bwd(const __nv_bfloat16 *__restrict__ dy, __nv_bfloat16 *dx, int B,
                                                   int NX, int NY, int NZ, int C, int accumulate) {
    const int64_t n = (int64_t)B * NX * NY * NZ * C;
    GRID_LOOP(q, n) {
        const int c = (int)(q % C);
        int64_t v = q / C;
        const int k = (int)(v % NZ); v /= NZ;
        const int j = (int)(v % NY); v /= NY;
        const int i = (int)(v % NX);
        const int b = (int)(v / NX);
        const int64_t cv = (((int64_t)b * (NX / 2) + i / 2) * (NY / 2) + j / 2) * (NZ / 2) + k / 2;
        float g = bf(dy[cv * C + c]) * 0.125f;
        if (accumulate) g += bf(dx[q]);
        dx[q] = __float2bfloat16_rn(g);
    }
}

// Nearest upsample (coarse -> fine).
__global__ void __launch_bounds__(256) k_up2(const __nv_bfloat16 *__restrict__ x, __nv_bfloat16 *__restrict__ y, int B,
                                             int NX, int NY, int NZ, int C) {
    const int64_t n = (int64_t)B * NX * NY * NZ * C;
    GRID_LOOP(q, n) {
        const int c = (int)(q % C);
        int64_t v = q / C;
        const int k = (int)(v % NZ); v /= NZ;
        const int j = (int)(v % NY); v /= NY;
        const int i = (int)(v % NX);
        const int b = (int)(v / NX);
        const int64_t cv = (((int64_t)b * (NX / 2) + i / 2) * (NY / 2) + j / 2) * (NZ / 2) + k / 2;
        y[q] = x[cv * C + c];
    }
}

// The same upsample for C % 8 == 0: thread t of fine row (b, i, j) copies
// channels 8 c8 .. 8 c8 + 7 of coarse voxel K into fine voxels 2K and 2K + 1
// (one 16-byte load, two 16-byte stores), with t = K * (C / 8) + c8.
// Grid: (ceil((NZ / 2) * (C / 8) / 128), NY, B * NX), 128 threads.
__global__ void __launch_bounds__(128) k_up2_v8(const uint4 *__restrict__ x, uint4 *__restrict__ y, int NX, int NY,
                                                int NZ, int C8) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int cz = NZ >> 1;
    if (t >= cz * C8) return;
    const int K = t / C8, c8 = t - K * C8;
    const int j = blockIdx.y, bi = blockIdx.z;
    const int b = bi / NX, i = bi - b * NX;
    const int64_t crow = ((int64_t)b * (NX >> 1) + (i >> 1)) * (NY >> 1) + (j >> 1);
    const uint4 v = __ldg(x + (crow * cz + K) * C8 + c8);
    const int64_t f = (((int64_t)bi * NY + j) * NZ + 2 * K) * C8 + c8;
    y[f] = v;
    y[f + C8] = v;
}

// Gradient of the upsample: dx_coarse = sum of the 8 fine gradients.
__global__ void __launch_bounds__(256) k_up2_bwd(const __nv_bfloat16 *__restrict__ dy, __nv_bfloat16 *__restrict__ dx,
                                                 int B, int NX, int NY, int NZ, int C) {
    const int cx = NX / 2, cy = NY / 2, cz = NZ / 2;
    const int64_t n = (int64_t)B * cx * cy * cz * C;
    GRID_LOOP(q, n) {
        const int c = (int)(q % C);
        int64_t v = q / C;
        const int k = (int)(v % cz); v /= cz;
        const int j = (int)(v % cy); v /= cy;
        const int i = (int)(v % cx);
        const int b = (int)(v / cx);
        float s = 0.0f;
        for (int d = 0; d < 8; d++) {
            const int64_t f = ((((int64_t)b * NX + 2 * i + (d >> 2)) * NY + 2 * j + ((d >> 1) & 1)) * NZ + 2 * k + (d & 1));
            s += bf(dy[f * C + c]);
        }
        dx[q] = __float2bfloat16_rn(s);
    }
}

// dx = dy where the ReLU output y > 0, else 0 (dx may alias dy).
__global__ void __launch_bounds__(256) k_relu_bwd(const __nv_bfloat16 *dy, const __nv_bfloat16 *__restrict__ y,
                                                  __nv_bfloat16 *dx, int64_t n) {
    GRID_LOOP(q, n) dx[q] = bf(y[q]) > 0.0f ? dy[q] : __float2bfloat16_rn(0.0f);
}

// 1x1x1 head: out[v] = sum_c w[c] x[v][c] + b, 16 channels, FP32 out.
__global__ void __launch_bounds__(256) k_head_fwd(const __nv_bfloat16 *__restrict__ x, const float *__restrict__ w,
                                                  const float *__restrict__ bias, float *__restrict__ out, int64_t n) {
    GRID_LOOP(v, n) {
        float s = bias[0];
#pragma unroll
        for (int c = 0; c < 16; c++) s = fmaf(w[c], bf(x[v * 16 + c]), s);
        out[v] = s;
    }
}

// Head gradients: dx[v][c] = dout[v] w[c]; dw[c] += sum_v dout[v] x[v][c]; db += sum dout.
__global__ void __launch_bounds__(256) k_head_bwd(const __nv_bfloat16 *__restrict__ x, const float *__restrict__ w,
                                                  const float *__restrict__ dout, __nv_bfloat16 *__restrict__ dx,
                                                  float *__restrict__ dw, float *__restrict__ db, int64_t n) {
    __shared__ double red[32];
    float acc[17];
#pragma unroll
    for (int c = 0; c < 17; c++) acc[c] = 0.0f;
    GRID_LOOP(v, n) {
        const float g = dout[v];
#pragma unroll
        for (int c = 0; c < 16; c++) {
            acc[c] = fmaf(g, bf(x[v * 16 + c]), acc[c]);
            dx[v * 16 + c] = __float2bfloat16_rn(g * w[c]);
        }
        acc[16] += g;
    }
    for (int c = 0; c < 17; c++) {
        const double t = block_sum((double)acc[c], red);
        if (threadIdx.x == 0) atomicAdd(c < 16 ? dw + c : db, (float)t);
    }
}

// Per-sample squared norm of the normalised target over fluid cells.
__global__ void __launch_bounds__(256) k_target_norm(const float *__restrict__ x, const int32_t *__restrict__ tag,
                                                     const float *__restrict__ inv_scale, int64_t ncell,
                                                     double *__restrict__ norm) {
    __shared__ double red[32];
    const int b = blockIdx.x;
    const float sc = inv_scale[b];
    double s = 0.0;
    for (int64_t q = threadIdx.x; q < ncell; q += blockDim.x) {
        const int64_t v = b * ncell + q;
        if (tag[v] == 1) {
            const double t = (double)(x[v] * sc);
            s += t * t;
        }
    }
    s = block_sum(s, red);
    if (threadIdx.x == 0) norm[b] = s;
}

// Masked MSE on fluid cells in normalised units: target = x * inv_scale[b].
// Weight per cell: inv_count, or 1 / (B * |target_b|^2) with per-sample norms
// (relative error averaged over the batch).  loss (FP64) and dpred.
__global__ void __launch_bounds__(256) k_unet_loss(const float *__restrict__ pred, const float *__restrict__ x,
                                                   const int32_t *__restrict__ tag, const float *__restrict__ inv_scale,
                                                   const double *__restrict__ norm, int B, int64_t ncell, int64_t n,
                                                   double inv_count, float *__restrict__ dpred,
                                                   double *__restrict__ loss) {
    __shared__ double red[32];
    double s = 0.0;
    GRID_LOOP(v, n) {
        float g = 0.0f;
        if (tag[v] == 1) {
            const int64_t b = v / ncell;
            const double w = norm ? (norm[b] > 0.0 ? 1.0 / (B * norm[b]) : 0.0) : inv_count;
            const float d = pred[v] - x[v] * inv_scale[b];
            s += w * ((double)d * d);
            g = (float)(2.0 * w) * d;
        }
        dpred[v] = g;
    }
    s = block_sum(s, red);
    if (threadIdx.x == 0) atomicAdd(loss, s);
}

// Network output (normalised) -> pressure guess: x0 = out / inv_scale * gain on
// fluid cells, 0 elsewhere.
__global__ void __launch_bounds__(256) k_unet_output(const float *__restrict__ out, const int32_t *__restrict__ tag,
                                                     const float *__restrict__ inv_scale, int64_t ncell, int64_t n,
                                                     float gain, float *__restrict__ x0) {
    GRID_LOOP(v, n) x0[v] = tag[v] == 1 ? out[v] / inv_scale[v / ncell] * gain : 0.0f;
}

// Bias gradient db[co] += sum_v dy[v][co]: each thread owns one 8-channel
// chunk (16 bytes) of the voxel rows it visits; per-block sums in shared
// memory, one global atomic per channel and block.
__global__ void __launch_bounds__(256) k_bias_grad(const uint4 *__restrict__ dy, int nch, int64_t nq,
                                                   float *__restrict__ db) {
    __shared__ float sb[64];
    if (threadIdx.x < 64) sb[threadIdx.x] = 0.0f;
    __syncthreads();
    float acc[8];
#pragma unroll
    for (int e = 0; e < 8; e++) acc[e] = 0.0f;
    // blockDim and the grid stride are multiples of nch: q % nch is fixed per thread
    GRID_LOOP(q, nq) {
        const uint4 u = dy[q];
        const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const float2 f = __bfloat1622float2(h[e]);
            acc[2 * e] += f.x;
            acc[2 * e + 1] += f.y;
        }
    }
    const int j = threadIdx.x % nch;
#pragma unroll
    for (int e = 0; e < 8; e++) atomicAdd(&sb[j * 8 + e], acc[e]);
    __syncthreads();
    if (threadIdx.x < nch * 8) atomicAdd(&db[threadIdx.x], sb[threadIdx.x]);
}

int launch_bias_grad(const void *dy, int cout, int64_t nvox, float *db, cudaStream_t s) {
    const int nch = cout / 8;
    const int64_t nq = nvox * nch;
    k_bias_grad<<<blocks_for(nq, 256, 152 * 8), 256, 0, s>>>(static_cast<const uint4 *>(dy), nch, nq, db);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

// Adam (decoupled weight decay off) on FP32 masters; optionally writes the BF16
// weights [27][cout][cin] and the flipped, transposed BF16 copy
// [27][cin][cout] (tap 26 - t) used by the data gradient.
__global__ void __launch_bounds__(256) k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                                              float *__restrict__ v, int64_t n, float lr, float b1, float b2,
                                              float eps, float c1, float c2, __nv_bfloat16 *__restrict__ w16,
                                              __nv_bfloat16 *__restrict__ w16t, int cout, int cin) {
    GRID_LOOP(q, n) {
        const float gq = g[q];
        const float mq = b1 * m[q] + (1.0f - b1) * gq;
        const float vq = b2 * v[q] + (1.0f - b2) * gq * gq;
        m[q] = mq;
        v[q] = vq;
        const float pq = p[q] - lr * (mq * c1) / (sqrtf(vq * c2) + eps);
        p[q] = pq;
        if (w16) {
            const int64_t tap = q / ((int64_t)cout * cin);
            const int co = (int)((q / cin) % cout), ci = (int)(q % cin);
            w16[q] = __float2bfloat16_rn(pq);
            w16t[((26 - tap) * cin + ci) * cout + co] = __float2bfloat16_rn(pq);
        }
    }
}

}  // namespace flub

using namespace flub;

static inline unsigned nb(int64_t n) { return blocks_for(n, 256, 152 * 16); }

extern "C" {

int flub_unet_input(const float *div, const int32_t *tag, int B, int64_t ncell, float *inv_scale, double *work,
                    void *out, void *stream) {
    FLUB_REQUIRE(div && tag && inv_scale && work && out && B > 0 && ncell > 0, "flub_unet_input: bad arguments");
    cudaStream_t s = as_stream(stream);
    const int parts = (int)((ncell + 255) / 256 < kRmsBlocks ? (ncell + 255) / 256 : kRmsBlocks);
    k_unet_rms_part<<<dim3(parts, B), 256, 0, s>>>(div, tag, ncell, work);
    FLUB_CHECK_LAUNCH();
    k_unet_rms_final<<<B, 256, 0, s>>>(work, parts, inv_scale);
    FLUB_CHECK_LAUNCH();
    const int64_t n = (int64_t)B * ncell;
    k_unet_input<<<nb(n), 256, 0, s>>>(div, tag, inv_scale, ncell, n, static_cast<__nv_bfloat16 *>(out));
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_pool2_bf16(const void *x, void *y, int B, int NX, int NY, int NZ, int C, void *stream) {
    FLUB_REQUIRE(x && y && NX % 2 == 0 && NY % 2 == 0 && NZ % 2 == 0, "flub_pool2_bf16: bad arguments");
    const bool v8 = C % 8 == 0 && (int64_t)B * (NX / 2) <= 65535 && NY / 2 <= 65535 &&
                    ((uintptr_t)x | (uintptr_t)y) % 16 == 0;
    if (v8) {
        const int C8 = C / 8, units = (NZ / 2) * C8;
        k_pool2_v8<<<dim3((unsigned)((units + 127) / 128), (unsigned)(NY / 2), (unsigned)(B * (NX / 2))), 128, 0,
                     as_stream(stream)>>>(static_cast<const uint4 *>(x), static_cast<uint4 *>(y), NX, NY, NZ, C8);
    } else {
        k_pool2<<<nb((int64_t)B * NX * NY * NZ * C / 8), 256, 0, as_stream(stream)>>>(
            static_cast<const __nv_bfloat16 *>(x), static_cast<__nv_bfloat16 *>(y), B, NX, NY, NZ, C);
    }
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_pool2_bwd_bf16(const void *dy, void *dx, int B, int NX, int NY, int NZ, int C, int accumulate, void *stream) {
    FLUB_REQUIRE(dy && dx, "flub_pool2_bwd_bf16: bad arguments");
    k_pool2_bwd<<<nb((int64_t)B * NX * NY * NZ * C), 256, 0, as_stream(stream)>>>(
        static_cast<const __nv_bfloat16 *>(dy), static_cast<__nv_bfloat16 *>(dx), B, NX, NY, NZ, C, accumulate);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_up2_bf16(const void *x, void *y, int B, int NX, int NY, int NZ, int C, void *stream) {
    FLUB_REQUIRE(x && y, "flub_up2_bf16: bad arguments");
    const bool v8 = C % 8 == 0 && NZ % 2 == 0 && (int64_t)B * NX <= 65535 && NY <= 65535 &&
                    ((uintptr_t)x | (uintptr_t)y) % 16 == 0;
    if (v8) {
        const int C8 = C / 8, units = (NZ / 2) * C8;
        k_up2_v8<<<dim3((unsigned)((units + 127) / 128), (unsigned)NY, (unsigned)(B * NX)), 128, 0,
                   as_stream(stream)>>>(static_cast<const uint4 *>(x), static_cast<uint4 *>(y), NX, NY, NZ, C8);
    } else {
        k_up2<<<nb((int64_t)B * NX * NY * NZ * C), 256, 0, as_stream(stream)>>>(
            static_cast<const __nv_bfloat16 *>(x), static_cast<__nv_bfloat16 *>(y), B, NX, NY, NZ, C);
    }
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_up2_bwd_bf16(const void *dy, void *dx, int B, int NX, int NY, int NZ, int C, void *stream) {
    FLUB_REQUIRE(dy && dx, "flub_up2_bwd_bf16: bad arguments");
    k_up2_bwd<<<nb((int64_t)B * NX * NY * NZ * C / 8), 256, 0, as_stream(stream)>>>(
        static_cast<const __nv_bfloat16 *>(dy), static_cast<__nv_bfloat16 *>(dx), B, NX, NY, NZ, C);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_relu_bwd_bf16(const void *dy, const void *y, void *dx, int64_t n, void *stream) {
    FLUB_REQUIRE(dy && y && dx, "flub_relu_bwd_bf16: bad arguments");
    k_relu_bwd<<<nb(n), 256, 0, as_stream(stream)>>>(static_cast<const __nv_bfloat16 *>(dy),
                                                     static_cast<const __nv_bfloat16 *>(y),
                                                     static_cast<__nv_bfloat16 *>(dx), n);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_head_fwd(const void *x, const float *w, const float *b, float *out, int64_t n, void *stream) {
    FLUB_REQUIRE(x && w && b && out, "flub_head_fwd: bad arguments");
    k_head_fwd<<<nb(n), 256, 0, as_stream(stream)>>>(static_cast<const __nv_bfloat16 *>(x), w, b, out, n);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_head_bwd(const void *x, const float *w, const float *dout, void *dx, float *dw, float *db, int64_t n,
                  void *stream) {
    FLUB_REQUIRE(x && w && dout && dx && dw && db, "flub_head_bwd: bad arguments");
    k_head_bwd<<<blocks_for(n, 256, 152 * 4), 256, 0, as_stream(stream)>>>(
        static_cast<const __nv_bfloat16 *>(x), w, dout, static_cast<__nv_bfloat16 *>(dx), dw, db, n);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_unet_loss(const float *pred, const float *x, const int32_t *tag, const float *inv_scale, int64_t ncell,
                   int B, double inv_count, double *sample_norm, float *dpred, double *loss, void *stream) {
    FLUB_REQUIRE(pred && x && tag && inv_scale && dpred && loss && B > 0, "flub_unet_loss: bad arguments");
    const int64_t n = (int64_t)B * ncell;
    cudaStream_t s = as_stream(stream);
    if (sample_norm) {
        k_target_norm<<<B, 256, 0, s>>>(x, tag, inv_scale, ncell, sample_norm);
        FLUB_CHECK_LAUNCH();
    }
    k_unet_loss<<<nb(n), 256, 0, s>>>(pred, x, tag, inv_scale, sample_norm, B, ncell, n, inv_count, dpred, loss);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_unet_output(const float *out, const int32_t *tag, const float *inv_scale, int64_t ncell, int B, float gain,
                     float *x0, void *stream) {
    FLUB_REQUIRE(out && tag && inv_scale && x0, "flub_unet_output: bad arguments");
    const int64_t n = (int64_t)B * ncell;
    k_unet_output<<<nb(n), 256, 0, as_stream(stream)>>>(out, tag, inv_scale, ncell, n, gain, x0);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

int flub_adam(float *p, const float *g, float *m, float *v, int64_t n, float lr, float b1, float b2, float eps,
              int step, void *w16, void *w16t, int cout, int cin, void *stream) {
    FLUB_REQUIRE(p && g && m && v && n > 0 && step > 0, "flub_adam: bad arguments");
    FLUB_REQUIRE(!w16 || ((int64_t)27 * cout * cin == n && w16t), "flub_adam: weight shape mismatch");
    const float c1 = 1.0f / (1.0f - powf(b1, (float)step)), c2 = 1.0f / (1.0f - powf(b2, (float)step));
    k_adam<<<nb(n), 256, 0, as_stream(stream)>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2,
                                                 static_cast<__nv_bfloat16 *>(w16), static_cast<__nv_bfloat16 *>(w16t),
                                                 cout, cin);
    FLUB_CHECK_LAUNCH();
    return FLUB_OK;
}

}  // extern "C"
