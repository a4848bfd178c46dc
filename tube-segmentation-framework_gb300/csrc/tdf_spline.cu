// tdf_spline.cu -- the spline tube detection filter (reference splineTDF,
// kernels.cl:1159-1254 and kernels_no_3d_write.cl:1574-1671; driver
// runSplineTDF, tubeDetectionFilters.cpp:4-55), used instead of the
// circle-fitting TDF by the presets with `use-spline-tdf`.
//
// Per voxel: the Hessian of the normalised field (gradientNormalized) and its
// eigen-decomposition, as in the circle-fitting TDF; then 12 arms in the plane
// of e2 and e3 (arm j at angle 2 pi j / 12).  Each arm searches outwards from
// rMin in steps of rStep for a border point: the field magnitude has risen at
// least once (or did not fall from the voxel to rMin), now falls, and the mean
// of the last two magnitudes exceeds the voxel's own by 0.1.  A voxel whose
// arm finds no border point, or whose border field points along the arm, is
// invalid (T = 0).  Otherwise T = min(1, mean(1 - |dir . e1|) * symmetry + 0.2)
// where symmetry averages min/max of the radii of opposite arms; R is the
// arms' radius sum / 12 (also for invalid voxels, over the arms searched).
//
// One thread per voxel, blocks of 8 x 4 x 4 voxels so that a block's samples
// stay in a small neighbourhood (L1).  Samples use the OpenCL linear sampler
// (tdf_common.cuh); voxels whose every sample corner lies inside the volume
// take the unclamped sampler, which gives the same bits.
#include "tdf_common.cuh"

namespace tsf {

constexpr int kArms = 12;
// Upper bound on the radii one arm evaluates (a radius step of 0, or one lost
// against the radius in float, would otherwise never end the search).
constexpr int kSplineMaxRadii = 4096;
// minAverageMag of the reference's driver (tubeDetectionFilters.cpp:47).
constexpr float kMinAverageMag = 0.1f;

struct ArmTable {
    float c[kArms];
    float s[kArms];
};

// alpha_j = 2 * M_PI_F * j / 12 in float (M_PI_F = the float nearest pi);
// cos and sin evaluated in double and rounded to float.
static ArmTable host_arm_table() {
    ArmTable t;
    const float two_pi = 2.0f * 3.14159265358979323846f;
    for (int j = 0; j < kArms; j++) {
        const float alpha = two_pi * (float)j / (float)kArms;
        t.c[j] = (float)std::cos((double)alpha);
        t.s[j] = (float)std::sin((double)alpha);
    }
    return t;
}

__device__ __forceinline__ float len3(float a, float b, float c) { return sqrtf((a * a + b * b) + c * c); }

template <int ST, bool INSIDE>
__device__ __forceinline__ float3 spline_sample(const void *F, int X, int Y, int Z, float u, float v, float w) {
    if (INSIDE) return sample_linear_in<ST>(F, X, X * Y, u, v, w);
    return sample_linear<ST>(F, X, Y, Z, u, v, w);
}

// One voxel's filter; INSIDE: every sample corner lies in the volume.
template <int ST, bool INSIDE>
__device__ __forceinline__ void spline_voxel(const void *F, int X, int Y, int Z, int x, int y, int z, float rmin,
                                             float rmax, float rstep, const ArmTable &tab, const float V[3][3],
                                             float cur, float &T, float &R) {
    const float e1x = V[0][0], e1y = V[1][0], e1z = V[2][0];
    const float e2x = V[0][1], e2y = V[1][1], e2z = V[2][1];
    const float e3x = V[0][2], e3y = V[1][2], e3z = V[2][2];
    const float fx = (float)x, fy = (float)y, fz = (float)z;
    float mr[kArms];
    float sum = 0.0f, avg = 0.0f;
    bool invalid = false;
    for (int j = 0; j < kArms; j++) {
        mr[j] = 999.0f;
        const float c = tab.c[j], s = tab.s[j];
        const float va0 = c * e3x + s * e2x, va1 = c * e3y + s * e2y, va2 = c * e3z + s * e2z;
        const float3 p0 = spline_sample<ST, INSIDE>(F, X, Y, Z, fx + rmin * va0, fy + rmin * va1, fz + rmin * va2);
        float prev = len3(p0.x, p0.y, p0.z);
        bool up = !(cur > prev);
        int nr = 0;
        for (float radius = rmin + rstep; radius <= rmax && nr < kSplineMaxRadii; radius = radius + rstep, nr++) {
            const float3 v =
                spline_sample<ST, INSIDE>(F, X, Y, Z, fx + radius * va0, fy + radius * va1, fz + radius * va2);
            const float mag = len3(v.x, v.y, v.z);
            if (up && mag < prev && (prev + mag) / 2.0f - cur > kMinAverageMag) {
                mr[j] = radius;
                avg = avg + radius;
                const float nx = v.x / mag, ny = v.y / mag, nz = v.z / mag;
                const float la = len3(va0, va1, va2);
                const float ax = -(va0 / la), ay = -(va1 / la), az = -(va2 / la);
                if ((nx * ax + ny * ay) + nz * az < 0.0f) {
                    invalid = true;
                    sum = 0.0f;
                }
                sum = sum + (1.0f - fabsf((nx * e1x + ny * e1y) + nz * e1z));
                break;
            }
            if (mag > prev) up = true;
            prev = mag;
        }
        if (mr[j] == 999.0f || invalid) {
            invalid = true;
            break;
        }
    }
    R = avg / (float)kArms;
    if (invalid) {
        T = 0.0f;
        return;
    }
    float sym = 0.0f;
    for (int j = 0; j < kArms / 2; j++) sym = sym + fminf(mr[j], mr[kArms / 2 + j]) / fmaxf(mr[j], mr[kArms / 2 + j]);
    sym = sym / (float)(kArms / 2);
    T = fminf(1.0f, (sum / (float)kArms) * sym + 0.2f);
}

constexpr int kSpBX = 8, kSpBY = 4, kSpBZ = 4;

template <int ST, bool UNORM>
__global__ void __launch_bounds__(kSpBX *kSpBY *kSpBZ)
    tdf_spline_kernel(const void *__restrict__ F, int X, int Y, int Z, float rmin, float rmax, float rstep,
                      const ArmTable tab, int margin, int fast_ok, void *T, float *__restrict__ Rout) {
    const int x = blockIdx.x * kSpBX + threadIdx.x;
    const int y = blockIdx.y * kSpBY + threadIdx.y;
    const int z = blockIdx.z * kSpBZ + threadIdx.z;
    if (x >= X || y >= Y || z >= Z) return;
    float H[3][3], V[3][3], d[3];
    hessian<ST, true>(F, X, Y, Z, x, y, z, H);
    eig3<float>(H, V, d);
    const int64_t i = lin(x, y, z, X, Y);
    const float4 c4 = Vec4Load<ST>::load(F, i);
    const float cur = len3(c4.x, c4.y, c4.z);
    const float e2[3] = {V[0][1], V[1][1], V[2][1]}, e3[3] = {V[0][2], V[1][2], V[2][2]};
    float t, r;
    if (fast_ok && samples_inside(x, y, z, X, Y, Z, margin, e2, e3))
        spline_voxel<ST, true>(F, X, Y, Z, x, y, z, rmin, rmax, rstep, tab, V, cur, t, r);
    else
        spline_voxel<ST, false>(F, X, Y, Z, x, y, z, rmin, rmax, rstep, tab, V, cur, t, r);
    if (UNORM) reinterpret_cast<uint16_t *>(T)[i] = to_unorm16(t);
    else reinterpret_cast<float *>(T)[i] = t;
    Rout[i] = r;
}

int run_tdf_spline(const void *F, int X, int Y, int Z, int st, float rmin, float rmax, float rstep, void *T, int unorm,
                   float *R, cudaStream_t s) {
    int rc = check_dims(X, Y, Z);
    if (rc) return rc;
    if (!valid_storage(st)) return fail(TSF_ERR_INVALID_ARG, "unknown storage format");
    if (!F || !T || !R) return fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (!(rmin == rmin) || !(rmax == rmax) || !(rstep == rstep))
        return fail(TSF_ERR_INVALID_ARG, "radius range is NaN");
    if (Z > 65535 * kSpBZ || Y > 65535 * kSpBY) return fail(TSF_ERR_INVALID_ARG, "volume too large for the grid");
    rmin = fmaxf(1.0f, rmin);   // runSplineTDF passes max(1, radiusMin)
    const ArmTable tab = host_arm_table();
    // the unclamped sampler needs 32-bit corner offsets and a finite margin
    const int fast_ok = ((int64_t)X * Y * Z < ((int64_t)1 << 31) - 1) && fmaxf(rmin, rmax) < 1.0e6f ? 1 : 0;
    const int margin = fast_ok ? sample_margin(fmaxf(rmin, rmax)) : 0;   // the first sample lies at rmin
    const dim3 blk(kSpBX, kSpBY, kSpBZ), grd((X + kSpBX - 1) / kSpBX, (Y + kSpBY - 1) / kSpBY, (Z + kSpBZ - 1) / kSpBZ);
    TSF_DISPATCH_STORAGE(st, ST, {
        if (unorm)
            tdf_spline_kernel<ST, true><<<grd, blk, 0, s>>>(F, X, Y, Z, rmin, rmax, rstep, tab, margin, fast_ok, T, R);
        else
            tdf_spline_kernel<ST, false><<<grd, blk, 0, s>>>(F, X, Y, Z, rmin, rmax, rstep, tab, margin, fast_ok, T, R);
    });
    TSF_CHECK_LAUNCH("tdf_spline_kernel");
    return TSF_OK;
}

}  // namespace tsf

extern "C" int tsf_tdf_spline(const void *d_field4, int X, int Y, int Z, int storage, float rmin, float rmax,
                              float rstep, void *d_T, int tdf_unorm16, float *d_R, void *stream) {
    return tsf::run_tdf_spline(d_field4, X, Y, Z, storage, rmin, rmax, rstep, d_T, tdf_unorm16, d_R,
                               reinterpret_cast<cudaStream_t>(stream));
}
