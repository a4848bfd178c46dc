/*
 * tsf_oracle.h -- CPU restatement of the Tube Segmentation Framework hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the CUDA
 * kernels of libtsf_gb300: only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py load it.  The product library never
 * links it and has no CPU fallback.
 *
 * Parity status: UNPINNED against outputs of the reference itself.  The
 * reference is OpenCL 1.1 code; it cannot be built or run here (no OpenCL
 * headers or platform, un-vendored SIPL / OpenCLUtilityLibrary submodules,
 * no Boost.iostreams, no GTest) and it ships no golden vectors.  Each function
 * below restates one reference kernel (file:line given beside it) step by step;
 * OpenCL image-sampler and format-conversion semantics follow the OpenCL 1.1
 * specification.  What is pinned: the eigen-solver against numpy's eigh, the
 * HP traversal order against a key sort, the storage conversions against
 * numpy, and the end-to-end centerpoint quality on the reference's own
 * synthetic test volume (tests/data/synthetic/dataset_1) when it is present,
 * and the whole run() chain passes the reference's system-test gates there.
 *
 * Every routine exists in two precisions: suffix _f32 (float arithmetic, the
 * same operation order as the CUDA kernels, compiled with -ffp-contract=off)
 * and _f64 (double arithmetic, no storage quantisation: the FP64 oracle).
 *
 * Volume layout: x fastest, index = x + X*(y + Y*z) (reference LPOS,
 * kernels.cl:9).  "field4" arrays are RGBA interleaved (x, y, z, w) per voxel,
 * matching the reference's CL_RGBA images; "planar" arrays are three
 * consecutive planes of N values (component-major).
 */
#ifndef TSF_ORACLE_H
#define TSF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Storage formats of vector fields (reference: CL_FLOAT or CL_SNORM_INT16,
 * tube-segmentation.cpp:417-423; FP16 / BF16 are additions of this library). */
enum { ORC_F32 = 0, ORC_F16 = 1, ORC_BF16 = 2, ORC_SNORM16 = 3 };

/* ---- storage conversions (float in, float out = value after a store+load) */
float orc_quantize(float x, int storage);
uint16_t orc_f32_to_f16_bits(float x);
float orc_f16_bits_to_f32(uint16_t h);
uint16_t orc_f32_to_bf16_bits(float x);
int16_t orc_f32_to_snorm16(float x);      /* convert_short_sat_rte(x*32767) */
float orc_snorm16_to_f32(int16_t s);      /* max(-1, s/32767)               */
uint16_t orc_f32_to_unorm16(float x);     /* convert_ushort_sat_rte(x*65535)*/
float orc_unorm16_to_f32(uint16_t u);     /* u/65535                        */
void orc_quantize_array(float *a, int64_t n, int storage);
void orc_to_unorm16_array(const float *in, uint16_t *out, int64_t n);
void orc_from_unorm16_array(const uint16_t *in, float *out, int64_t n);

/* cos(j), sin(j) for j = 0..31 radians rounded to 6 significant digits, the
 * sample directions of circleFittingTDF (kernels.cl:1068-1069). */
void orc_circle_table(float cosv[32], float sinv[32]);

/* The 12 arm directions of splineTDF (kernels.cl:1211-1212): alpha_j =
 * 2 * M_PI_F * j / 12 in float, cos and sin in double rounded to float. */
void orc_arm_table(float cosv[12], float sinv[12]);

/* createBlurMask (tube-segmentation.cpp:188-211).  mask must hold 11^3 floats.
 * Returns maskSize (the half width m). */
int orc_blur_mask(float sigma, float *mask);

/* ---- histogram-pyramid compaction (kernels.cl:63-299, oul HP host class).
 * Builds the pyramid over mask (0/1 bytes) and enumerates positions in the
 * pyramid's traversal order.  Returns the number of set voxels; writes up to
 * cap positions (int3 each) to pos. */
int64_t orc_hp_compact(const int8_t *mask, int X, int Y, int Z, int32_t *pos, int64_t cap);

/* ---- templated kernels: see tsf_oracle_impl.h for the list */
#define ORC_DECLARE(R, S)                                                               \
    void orc_blur##S(const float *in, int X, int Y, int Z, int m, const float *mask,     \
                     R *out);                                                           \
    void orc_vector_field##S(const R *in, int X, int Y, int Z, float Fmax, int vsign,    \
                             int storage, R *field4);                                   \
    void orc_gvf_init##S(const R *field4, int64_t n, R *v_planar, R *f_planar);         \
    void orc_gvf##S(const R *f_planar, R *v_planar, int X, int Y, int Z, float mu,       \
                    int iterations, int storage);                                       \
    void orc_gvf_finish##S(const R *v_planar, int64_t n, int storage, R *field4);       \
    void orc_gvf_one_component##S(const R *field4, int X, int Y, int Z, float mu,        \
                                  int iterations, int storage, R *out4);                \
    void orc_eig3##S(const R A[9], R V[9], R d[3]);                                     \
    void orc_tdf_circle##S(const R *field4, int X, int Y, int Z, float rMin, float rMax,  \
                           float rStep, R *T, R *radius);                               \
    void orc_tdf_circle_ex##S(const R *field4, int X, int Y, int Z, float rMin, float rMax, \
                              float rStep, int samples, int stride, int eigen, R *T,     \
                              R *radius);                                               \
    void orc_tdf_spline##S(const R *field4, int X, int Y, int Z, float rMin, float rMax,  \
                           float rStep, R *T, R *radius);                               \
    void orc_combine##S(const R *Ts, const R *Rs, R *Tl, R *Rl, int64_t n);             \
    void orc_candidates2##S(const R *radius, const R *field4, int X, int Y, int Z,       \
                            const int32_t *pos, int64_t count, int8_t *mask_out);       \
    void orc_dd##S(const R *T, const int8_t *cand, int X, int Y, int Z, int cubeSize,    \
                   int8_t *out);                                                        \
    void orc_fmg_gvf##S(const R *field4, int X, int Y, int Z, float mu, int iterations,  \
                        int storage, R *out4);

ORC_DECLARE(float, _f32)
ORC_DECLARE(double, _f64)

/* GVF residual norms (no reference counterpart: the reference never reduces
 * its residuals).  Per component c, at the mirrored position of every voxel,
 * in float in the reference's operation order:
 *   kind 0 (GVF3DIteration's update, kernels.cl:1486-1490):
 *     r = mu * L(v_c) - (v_c - f0_c) |f0|^2
 *   kind 1 (fmgResidual, kernels.cl:2008-2053, spacing 1):
 *     r = -|f0|^2 f0_c - (mu * (sum of 6 neighbours - 6 v_c) - |f0|^2 v_c)
 * f0 and v planar [3][Z][Y][X] (stored values).  out[0..2] = sqrt(sum r_c^2)
 * (squares and sums in double), out[3] = sqrt of the total, out[4] = max |r|. */
void orc_gvf_residual_norm(const float *f0, const float *v, int X, int Y, int Z, float mu, int kind, double out[5]);

/* The closed-form eigensolver of the TDF's eigen mode 1 (tsf_oracle_eigc.h,
 * no reference counterpart): A row-major symmetric, V columns = eigenvectors
 * (largest component positive), d ascending by |lambda|. */
void orc_eig3_closed_f32(const float A[9], float V[9], float d[3]);

/* threshold (findCandidateCenterpoints, kernels.cl:1296-1307) */
void orc_threshold_f32(const float *T, int64_t n, float thr, int8_t *mask);

/* Threads used by the OpenMP loops (0 = library default). */
void orc_set_threads(int n);

/* centerline linking (parallelCenterlineExtraction.cpp:911-1332,
 * kernels.cl:327-559): returns the edge count; edges (capacity 2n pairs) in
 * the 2-D pyramid order, labels = smallest vertex index of the component,
 * sizes indexed by label. */
int orc_link_centerpoints(const int32_t *v, int n, const float *T, int X, int Y, int Z, float min_avg, float maxd,
                          int32_t *edges, int32_t *labels, int32_t *sizes);
/* removeSmallTrees (kernels.cl:510-534): rasterise edges of trees of at least
 * min_tree vertices into out (X*Y*Z int8, not cleared) */
void orc_rasterize_trees(const int32_t *v, const int32_t *edges, int ne, const int32_t *labels,
                         const int32_t *sizes, int min_tree, int8_t *out, int X, int Y, int Z);
int orc_get_threads(void);

/* Raw voxel types (the reference's MET_* element types). */
enum { ORC_RAW_U8 = 0, ORC_RAW_I8 = 1, ORC_RAW_U16 = 2, ORC_RAW_I16 = 3, ORC_RAW_F32 = 4 };
/* cropDatasetThreshold (method 0) / cropDatasetLung (method 1), kernels.cl:813-946:
 * per-slice counts of inside scan lines, X + Y + Z int16 (x slices, y, z). */
void orc_crop_scan_lines(const void *vol, int type, int X, int Y, int Z, int method, float threshold,
                         int16_t *counts);

/* runInverseGradientSegmentation (segmentation.cpp:5-205): grows from the
 * centerline (initGrowing, grow; each iteration decides, then applies with the
 * precedence accepted > to check > dropped), closes (dilate, erode) into out
 * (X*Y*Z int8, written).  field4 as read (float).  Returns the number of grow
 * iterations, the last of which accepted nothing. */
int orc_segment_inverse_gradient(const int8_t *cl, const float *field4, const float *radius, int X, int Y, int Z,
                                 int8_t *out);
/* runSphereSegmentation (segmentation.cpp:207-307) into out (written) */
void orc_segment_spheres(const int8_t *cl, const float *radius, int X, int Y, int Z, int8_t *out);

#ifdef __cplusplus
}
#endif
#endif
