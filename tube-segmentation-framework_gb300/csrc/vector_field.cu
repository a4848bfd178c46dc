// vector_field.cu -- the GVF input stage: Gaussian blur and the normalised
// gradient field f0 (reference: blurVolumeWithGaussian / createVectorField,
// kernels.cl:1017-1063; createBlurMask, tube-segmentation.cpp:188-211).
//
// Both kernels are one thread per voxel over x-fastest volumes.  The blur
// mask travels as a by-value kernel parameter (at most 11^3 floats), so every
// warp reads it from the constant bank with a broadcast.  Reads of the float
// volume go through the read-only path; the x/y neighbours of a 32x4x2 block
// hit L1.  HBM traffic is 8 B/voxel for the blur and 4 + 3s (+4s with the
// field4 image) bytes/voxel for the vector field.
#include <math.h>

#include "tsf_common.cuh"

namespace tsf {

struct BlurMask {
    float w[1331];
    int m;
};

// createBlurMask (tube-segmentation.cpp:188-211): half width ceil(sigma/0.5)
// clamped to [1,5]; the exponential is evaluated in double and rounded to
// float, the normalising sum is kept in float.
int host_blur_mask(float sigma, float *mask, int *half_width) {
    if (!(sigma > 0.0f)) return fail(TSF_ERR_INVALID_ARG, "blur sigma must be > 0");
    int m = (int)ceilf(sigma / 0.5f);
    if (m < 1) m = 1;
    if (m > 5) m = 5;
    const int S = 2 * m + 1;
    float sum = 0.0f;
    const float two_s2 = (2.0f * sigma) * sigma;
    for (int a = -m; a <= m; a++)
        for (int b = -m; b <= m; b++)
            for (int c = -m; c <= m; c++) {
                volatile float arg = -((float)(a * a + b * b + c * c) / two_s2);
                double w = exp((double)arg);
                sum = (float)((double)sum + w);
                mask[(a + m) + (b + m) * S + (c + m) * S * S] = (float)w;
            }
    for (int i = 0; i < S * S * S; i++) mask[i] = mask[i] / sum;
    *half_width = m;
    return TSF_OK;
}

__global__ void __launch_bounds__(256) blur_kernel(const float *__restrict__ in, float *__restrict__ out,
                                                   int X, int Y, int Z, const BlurMask mask) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= X || y >= Y || z >= Z) return;
    const int m = mask.m, S = 2 * m + 1;
    float sum = 0.0f;
    for (int c = -m; c <= m; c++) {
        const int zz = clampi(z + c, Z);
        for (int b = -m; b <= m; b++) {
            const int yy = clampi(y + b, Y);
            const float *row = in + lin(0, yy, zz, X, Y);
            const float *wrow = mask.w + (b + m) * S + (c + m) * S * S + m;
            for (int a = -m; a <= m; a++) {
                sum = sum + wrow[a] * __ldg(row + clampi(x + a, X));
            }
        }
    }
    out[lin(x, y, z, X, Y)] = sum;
}

// The same blur with the half width fixed at compile time: voxels whose
// (2M+1)^3 neighbourhood lies inside the volume take fully unrolled loops (the
// weights become constant operands, the row offsets immediates, no clamps);
// the others take the clamped loops.  Same weights, same order (z outer, then
// y, then x), so the same bits as blur_kernel.
template <int M>
__global__ void __launch_bounds__(256) blur_m_kernel(const float *__restrict__ in, float *__restrict__ out,
                                                     int X, int Y, int Z, const BlurMask mask) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= X || y >= Y || z >= Z) return;
    constexpr int S = 2 * M + 1;
    float sum = 0.0f;
    if (x >= M && x + M < X && y >= M && y + M < Y && z >= M && z + M < Z) {
        const float *base = in + lin(x, y, z, X, Y);
        const int64_t sy = X, sz = (int64_t)X * Y;
#pragma unroll
        for (int c = -M; c <= M; c++) {
#pragma unroll
            for (int b = -M; b <= M; b++) {
                const float *row = base + c * sz + b * sy;
#pragma unroll
                for (int a = -M; a <= M; a++) sum = sum + mask.w[(a + M) + (b + M) * S + (c + M) * S * S] * __ldg(row + a);
            }
        }
    } else {
        for (int c = -M; c <= M; c++) {
            const int zz = clampi(z + c, Z);
            for (int b = -M; b <= M; b++) {
                const float *row = in + lin(0, clampi(y + b, Y), zz, X, Y);
                const float *wrow = mask.w + (b + M) * S + (c + M) * S * S + M;
                for (int a = -M; a <= M; a++) sum = sum + wrow[a] * __ldg(row + clampi(x + a, X));
            }
        }
    }
    out[lin(x, y, z, X, Y)] = sum;
}

template <int ST>
__global__ void __launch_bounds__(256) vector_field_kernel(const float *__restrict__ in, int X, int Y, int Z,
                                                           float fmax, float sg, void *planar, void *field4) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= X || y >= Y || z >= Z) return;
    const float gx = 0.5f * (__ldg(in + lin(clampi(x + 1, X), y, z, X, Y)) - __ldg(in + lin(clampi(x - 1, X), y, z, X, Y)));
    const float gy = 0.5f * (__ldg(in + lin(x, clampi(y + 1, Y), z, X, Y)) - __ldg(in + lin(x, clampi(y - 1, Y), z, X, Y)));
    const float gz = 0.5f * (__ldg(in + lin(x, y, clampi(z + 1, Z), X, Y)) - __ldg(in + lin(x, y, clampi(z - 1, Z), X, Y)));
    float Fx = sg * gx, Fy = sg * gy, Fz = sg * gz;
    const float l = sqrtf((Fx * Fx + Fy * Fy) + Fz * Fz);
    if (l < fmax) {
        Fx = Fx / fmax; Fy = Fy / fmax; Fz = Fz / fmax;
    } else {
        Fx = Fx / l; Fy = Fy / l; Fz = Fz / l;
    }
    const int64_t i = lin(x, y, z, X, Y);
    const int64_t n = (int64_t)X * Y * Z;
    using T = typename Store<ST>::T;
    if (planar) {
        T *p = reinterpret_cast<T *>(planar);
        p[i] = Store<ST>::store(Fx);
        p[n + i] = Store<ST>::store(Fy);
        p[2 * n + i] = Store<ST>::store(Fz);
    }
    if (field4) store4<ST>(field4, i, Fx, Fy, Fz, 1.0f);
}

static dim3 vox_block() { return dim3(32, 4, 2); }
static dim3 vox_grid(int X, int Y, int Z) {
    dim3 b = vox_block();
    return dim3((X + b.x - 1) / b.x, (Y + b.y - 1) / b.y, (Z + b.z - 1) / b.z);
}

int launch_blur(const float *d_in, float *d_out, int X, int Y, int Z, float sigma, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!d_in || !d_out) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (d_in == d_out) return fail(TSF_ERR_INVALID_ARG, "blur cannot run in place");
    BlurMask mask;
    r = host_blur_mask(sigma, mask.w, &mask.m);
    if (r) return r;
    const dim3 g = vox_grid(X, Y, Z), b = vox_block();
    switch (mask.m) {
    case 1: blur_m_kernel<1><<<g, b, 0, s>>>(d_in, d_out, X, Y, Z, mask); break;
    case 2: blur_m_kernel<2><<<g, b, 0, s>>>(d_in, d_out, X, Y, Z, mask); break;
    case 3: blur_m_kernel<3><<<g, b, 0, s>>>(d_in, d_out, X, Y, Z, mask); break;
    case 4: blur_m_kernel<4><<<g, b, 0, s>>>(d_in, d_out, X, Y, Z, mask); break;
    case 5: blur_m_kernel<5><<<g, b, 0, s>>>(d_in, d_out, X, Y, Z, mask); break;
    default: blur_kernel<<<g, b, 0, s>>>(d_in, d_out, X, Y, Z, mask); break;
    }
    TSF_CHECK_LAUNCH("blur_kernel");
    return TSF_OK;
}

int launch_vector_field(const float *d_in, int X, int Y, int Z, float fmax, int vsign, int st,
                        void *d_planar, void *d_field4, cudaStream_t s) {
    int r = check_dims(X, Y, Z);
    if (r) return r;
    if (!d_in || (!d_planar && !d_field4)) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (!(fmax > 0.0f)) return fail(TSF_ERR_INVALID_ARG, "fmax must be > 0");
    if (vsign != 1 && vsign != -1) return fail(TSF_ERR_INVALID_ARG, "vsign must be +1 or -1");
    const float sg = (float)vsign;
    TSF_DISPATCH_STORAGE(st, ST,
        vector_field_kernel<ST><<<vox_grid(X, Y, Z), vox_block(), 0, s>>>(d_in, X, Y, Z, fmax, sg, d_planar, d_field4));
    TSF_CHECK_LAUNCH("vector_field_kernel");
    return TSF_OK;
}

}  // namespace tsf
