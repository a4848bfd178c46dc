/*
 * tsf_c.h -- C ABI of libtsf_gb300, the GB300 (sm_103a) implementation of the
 * Tube Segmentation Framework's data-parallel hot path: gradient vector flow
 * (GVF), the fused Hessian / eigen-decomposition / circle-fitting tube
 * detection filter (TDF), and candidate-centerpoint compaction.
 *
 * Conventions
 *  - Every pointer argument named d_* is DEVICE memory on the current CUDA
 *    device, allocated by the caller.  No entry point allocates memory that
 *    the caller can see; scratch memory comes from a caller-provided workspace
 *    whose size is returned by the matching *_workspace_size query.
 *  - Volumes are X*Y*Z voxels, x fastest: index = x + X*(y + Y*z), the LPOS
 *    layout of the reference (kernels.cl:9).
 *  - "field4" buffers hold 4 interleaved components per voxel (x, y, z, w) in
 *    the given storage format, like the reference's CL_RGBA images.  "planar"
 *    buffers hold 3 consecutive planes of N = X*Y*Z values (x plane, y plane,
 *    z plane).
 *  - `stream` is a cudaStream_t (0 = legacy default stream).  Calls are
 *    stream-ordered and asynchronous unless documented otherwise, and are
 *    reentrant given distinct buffers and workspaces.
 *  - Return value: TSF_OK or an error code; tsf_last_error_string() gives the
 *    message of the calling thread's last failure.
 *  - Minimum extent: 4 voxels per axis (the reference shrinks volumes to a
 *    multiple of 4 per axis, tube-segmentation.cpp:1800-1828).
 *
 * Each entry point names the reference interface it replaces (paths relative
 * to the smistad/Tube-Segmentation-Framework source tree).  The reference's
 * stage signatures take cl::Image3D / cl::Buffer objects and an OpenCL
 * context, so they cannot be ABI-compatible; these functions take plain
 * device pointers and sizes instead.
 */
#ifndef TSF_C_H
#define TSF_C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TSF_ABI_VERSION 1

/* Status codes. */
enum {
    TSF_OK = 0,
    TSF_ERR_INVALID_ARG = 1,   /* bad dimensions, parameters or null pointers   */
    TSF_ERR_CUDA = 2,          /* a CUDA runtime call or kernel launch failed   */
    TSF_ERR_WORKSPACE = 3,     /* workspace smaller than *_workspace_size()     */
    TSF_ERR_COUNT_RANGE = 4,   /* candidate / vertex count outside the range
                                  the reference accepts
                                  (parallelCenterlineExtraction.cpp:842-844,
                                  895-899)                                      */
    TSF_ERR_NOT_CONVERGED = 5, /* an iteration cap was reached                  */
    TSF_ERR_CAPACITY = 6       /* an output buffer is too small, or the volume
                                  exceeds tsf_gvf_static's fixed scratch array  */
};

/* Storage formats of vector fields.  F32 and SNORM16 are the reference's
 * 32-bit and 16-bit options (CL_FLOAT / CL_SNORM_INT16,
 * tube-segmentation.cpp:417-423, gradientVectorFlow.cpp:1100-1106); F16 and
 * BF16 are additional 16-bit formats.  Arithmetic is always FP32. */
enum {
    TSF_STORE_F32 = 0,
    TSF_STORE_F16 = 1,
    TSF_STORE_BF16 = 2,
    TSF_STORE_SNORM16 = 3
};

/* Version of this ABI (TSF_ABI_VERSION). */
int tsf_abi_version(void);

/* Message of the calling thread's last failed call ("" if none). */
const char *tsf_last_error_string(void);

/* Bytes per stored component for a storage format (4 or 2; 0 if invalid). */
size_t tsf_storage_bytes(int storage);

/* Number of CUDA kernels this library has launched in this process (all
 * threads, all devices).  Lets a caller count the launches of a call. */
unsigned long long tsf_kernel_launches(void);

/* ---------------------------------------------------------------------------
 * Input stage
 * ------------------------------------------------------------------------- */

/* Voxel types of raw input volumes (MET_UCHAR, MET_CHAR, MET_USHORT,
 * MET_SHORT, MET_FLOAT in the reference's .mhd reader,
 * tube-segmentation.cpp:1490-1536). */
enum {
    TSF_TYPE_UINT8 = 0,
    TSF_TYPE_INT8 = 1,
    TSF_TYPE_UINT16 = 2,
    TSF_TYPE_INT16 = 3,
    TSF_TYPE_FLOAT32 = 4
};

/* toFloat (kernels.cl:989-1015, enqueued at tube-segmentation.cpp:1833-1892):
 * v = clamp(v, minimum, maximum); d_out = (v - minimum) / (maximum - minimum),
 * for n voxels of the given TSF_TYPE_*. */
int tsf_to_float(const void *d_in, int type, int64_t n, float minimum, float maximum, float *d_out,
                 void *stream);

/* Host helper: the normalised Gaussian blur mask of createBlurMask
 * (tube-segmentation.cpp:188-211).  mask_out must hold 11*11*11 floats; the
 * half width m (1..5) is written to *half_width. */
int tsf_blur_mask(float sigma, float *mask_out, int *half_width);

/* blurVolumeWithGaussian (kernels.cl:1017-1040, enqueued at
 * tube-segmentation.cpp:244-300 and 536-590): dense (2m+1)^3 Gaussian with
 * nearest clamp-to-edge reads.  d_in and d_out are float volumes and must not
 * overlap. */
int tsf_blur(const float *d_in, float *d_out, int X, int Y, int Z, float sigma, void *stream);

/* createVectorField (kernels.cl:1042-1063, enqueued at
 * tube-segmentation.cpp:301-443 and 603-730): F = vsign * grad(I) with the
 * Fmax normalisation.  Writes the planar f0 (3N elements) to d_planar and/or
 * the field4 image (4N elements, w = 1) to d_field4; either may be NULL. */
int tsf_vector_field(const float *d_in, int X, int Y, int Z, float fmax, int vsign, int storage,
                     void *d_planar, void *d_field4, void *stream);

/* ---------------------------------------------------------------------------
 * Gradient vector flow
 * ------------------------------------------------------------------------- */

/* Workspace bytes for tsf_gvf (one ping-pong copy of the planar field). */
size_t tsf_gvf_workspace_size(int X, int Y, int Z, int storage);

/* GVF Jacobi iterations: replaces runGVF / runFastGVF
 * (gradientVectorFlow.cpp:1007-1172, 1448-1457) with the GVF3DIteration
 * kernel (kernels.cl:1464-1493).  d_f0 is the planar initial field f0 (the
 * data term, read only); d_v holds the planar start value on entry (normally
 * a copy of f0, as GVF3DInit makes) and the result after exactly `iterations`
 * iterations on return.  mu is the GVF regularisation constant.  One
 * iteration per launch; every iteration's result is rounded to `storage`.
 * Note: the reference's host loop returns the result of iterations - 1 when
 * `iterations` is odd; the C++ layer (run()) reproduces that, this call does
 * not. */
int tsf_gvf(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int iterations,
            int storage, void *d_workspace, size_t workspace_bytes, void *stream);

/* tsf_gvf with the kernel chosen: 0 = the default of tsf_gvf (the
 * z-streaming kernel fed by TMA copies wherever rows are a multiple of 16
 * bytes and the buffers 16-byte aligned, else the register-vector kernel),
 * 1 = the register-vector (or per-voxel) kernel only, 2 = same as 0 with
 * every iteration streaming upwards, 3 = two iterations per launch (temporal
 * blocking: the first iteration's result stays in shared memory; volumes
 * with X >= 128, Y >= 8, Z >= 5 and 16-byte rows, else as 0; an odd count
 * ends with one launch of the default kernel).  All modes give
 * bit-identical results. */
int tsf_gvf_mode(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int iterations,
                 int storage, void *d_workspace, size_t workspace_bytes, int mode, void *stream);

/* Device-side error word of the streaming GVF kernels: 0 = none; bit 0 (the
 * forward kernel) or bit 1 (the adjoint kernel) = a shared-memory copy did not
 * complete within its wait limit (the kernel then stops early and its output
 * is invalid); -1 if the word could not be read.
 * clear != 0 resets the word.  Synchronises with the device.  No counterpart
 * in the reference (OpenCL reports no such condition). */
int tsf_gvf_device_error(int clear);

/* Self-test of the streaming GVF kernel's bounded waits (no counterpart in
 * the reference).  Launches the kernel once, on the caller's buffers as for
 * tsf_gvf (d_f0 read; d_v and the workspace of tsf_gvf_workspace_size bytes
 * receive invalid values), with every shared-memory copy suppressed and each
 * barrier wait limited to wait_cycles SM clock cycles (> 0; 2,000,000 is about
 * 1 ms): every wait runs out, the kernel records the timeout in its device
 * error word and returns, and the GPU stays usable.  Returns that error word
 * (as tsf_gvf_device_error(1) would: bit 0 set is the expected result), or
 * minus a TSF_ERR_* code when the kernel cannot run on these buffers (rows
 * not a multiple of 16 bytes, unaligned) or the launch fails.  Synchronises
 * `stream`. */
int tsf_gvf_wait_selftest(const void *d_f0, void *d_v, int X, int Y, int Z, int storage,
                          long long wait_cycles, void *d_workspace, size_t workspace_bytes, void *stream);

/* tsf_gvf for callers that cannot allocate device memory.  No counterpart in
 * the reference: it exists for hosts that can neither call cudaMalloc nor
 * provide a workspace (plug-in hosts that own the device allocator,
 * real-time pipelines that forbid device allocation once running).  Same
 * arguments and result as tsf_gvf, without the workspace: the scratch is a
 * fixed 96 MiB array in the library's device memory, held on every GPU that
 * loads the library until the process exits.  Limit: 3 * X*Y*Z stored
 * components must fit in 96 MiB (256^3 voxels in a 16-bit format, 8,388,608
 * in FP32); larger volumes return TSF_ERR_CAPACITY.  The first call on a
 * device looks up the array's address with that device current -- make it
 * before any stream capture; the address is kept for the process, so
 * cudaDeviceReset between calls is not supported.  All calls share the
 * array, so calls that overlap on the GPU race.  Allocates nothing. */
int tsf_gvf_static(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int iterations,
                   int storage, void *stream);

/* FP64 norms of the GVF residual (no counterpart in the reference, which
 * runs a fixed number of iterations and never reduces its residual images;
 * the per-voxel values are the reference's own).  Per component c, evaluated
 * in FP32 at the mirrored position of every voxel, in the reference's
 * operation order:
 *   kind 0 -- the Jacobi update of GVF3DIteration (kernels.cl:1486-1490),
 *             r_c = mu L(v_c) - (v_c - f0_c) |f0|^2, i.e. v_{k+1} - v_k before
 *             rounding to the storage format;
 *   kind 1 -- fmgResidual on the finest level (kernels.cl:2008-2053,
 *             spacing 1): r_c = -|f0|^2 f0_c - (mu L(v_c) - |f0|^2 v_c).
 * layout 0: d_f0 and d_v planar (tsf_gvf's buffers); 1: field4 (e.g.
 * tsf_gvf_fmg's input and output).  Squares are summed in FP64 in a fixed
 * order (the same bits on every run and device).  norms (host, 5 doubles):
 * sqrt(sum r_x^2), sqrt(sum r_y^2), sqrt(sum r_z^2), sqrt of the total, max
 * |r|.  Workspace: tsf_gvf_residual_workspace_size() bytes, 8-byte aligned.
 * Synchronises `stream`. */
size_t tsf_gvf_residual_workspace_size(void);
int tsf_gvf_residual_norm(const void *d_f0, const void *d_v, int X, int Y, int Z, float mu, int storage,
                          int kind, int layout, double *norms, void *d_workspace, size_t workspace_bytes,
                          void *stream);

/* Jacobi GVF (as tsf_gvf) that decides convergence on the residual: every
 * check_every iterations (and before the first) the RMS of the next update,
 * sqrt(sum_c |r_c|^2 / (3 N)) of tsf_gvf_residual_norm kind 0, is computed
 * in FP64; the call stops at the first check where it is <= tolerance.
 * *iterations_done and *residual_rms (host, may be NULL) receive the
 * iterations run and the last RMS.  TSF_ERR_NOT_CONVERGED when
 * max_iterations were run and the RMS is still above the tolerance (d_v then
 * holds the last iterate).  Synchronises `stream` at every check.  No
 * counterpart in the reference (fixed iteration count,
 * gradientVectorFlow.cpp:1137-1151). */
size_t tsf_gvf_converge_workspace_size(int X, int Y, int Z, int storage);
int tsf_gvf_converge(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int max_iterations,
                     int check_every, double tolerance, int storage, int *iterations_done,
                     double *residual_rms, void *d_workspace, size_t workspace_bytes, void *stream);

/* Converts n stored components from one storage format to another: each
 * value as it reads (e.g. max(-1, s / 32767) for snorm16) rounded to the
 * target format.  d_in and d_out must not overlap.  No counterpart in the
 * reference, whose fields keep one format; lets a caller continue a 16-bit
 * GVF in FP32 (tsf_gvf with FP32 storage from the converted iterate and an
 * FP32 f0) or store an FP32 field in 16 bits for the TDF. */
int tsf_convert_field(const void *d_in, int in_storage, void *d_out, int out_storage, int64_t n,
                      void *stream);

/* Workspace bytes for tsf_gvf_adjoint. */
size_t tsf_gvf_adjoint_workspace_size(int X, int Y, int Z, int storage, int iterations,
                                      int checkpoint_every);

/* Smallest checkpoint interval whose tsf_gvf_adjoint workspace fits in
 * budget_bytes: 1 keeps every forward state and recomputes nothing; 0 if no
 * interval fits.  No counterpart in the reference. */
int tsf_gvf_adjoint_checkpoint_interval(int X, int Y, int Z, int storage, int iterations,
                                        size_t budget_bytes);

/* Reverse-mode derivative of `iterations` GVF Jacobi iterations started from
 * v_0 = f0 (no counterpart in the reference, which has no derivatives).
 * Given d_gv = dL/dv_K (planar FP32), writes dL/df0 (planar FP32, all paths
 * through the data term, |f0|^2 and v_0) to d_gf0 and dL/dmu to *dmu (host,
 * FP64; NULL to skip -- otherwise the call synchronises `stream`).  Forward
 * states are recomputed from checkpoints kept every C = `checkpoint_every`
 * iterations (<= 0: ceil(sqrt(iterations))); the workspace holds about
 * K/C + C states (C = 1: all K-1 states, no recomputation).
 * flags bit 0: the checkpoints are already in the workspace
 * (tsf_gvf_checkpointed ran with the same arguments). */
int tsf_gvf_adjoint(const void *d_f0, int X, int Y, int Z, float mu, int iterations, int storage,
                    const float *d_gv, float *d_gf0, double *dmu, int checkpoint_every, int flags,
                    void *d_workspace, size_t workspace_bytes, void *stream);

/* Forward GVF that also stores the adjoint's checkpoints in the workspace of
 * tsf_gvf_adjoint (same sizes and interval); d_v (may be NULL) receives the
 * result after `iterations` iterations.  A following tsf_gvf_adjoint call with
 * flags bit 0 set reuses the checkpoints instead of recomputing them. */
int tsf_gvf_checkpointed(const void *d_f0, void *d_v, int X, int Y, int Z, float mu, int iterations,
                         int storage, int checkpoint_every, void *d_workspace,
                         size_t workspace_bytes, void *stream);

/* GVF3DFinish (kernels.cl:1506-1515): packs the planar field into a field4
 * image with w = |v| (1 where |v| == 0). */
int tsf_gvf_finish(const void *d_v, void *d_field4, int X, int Y, int Z, int storage,
                   void *stream);

/* The reference's low-memory GVF (runLowMemoryGVF, gradientVectorFlow.cpp:1172-1300,
 * kernels GVF3D{Init,Iteration,Finish}_one_component, kernels.cl:1392-1462 and
 * kernels_no_3d_write.cl:1669-1741; chosen by the reference when the RGBA field
 * exceeds the device's largest allocation, tube-segmentation.cpp:742-762): one
 * component at a time, with |f0|^2 stored in the field's format (rounded to it in
 * 16-bit formats), then the finish pass.  d_field4_in: the initial field4 image
 * (tsf_vector_field's d_field4); d_field4_out: the result with w = |v|.  Workspace
 * (6 N stored values) from tsf_gvf_one_component_workspace_size.  With FP32
 * storage the result equals tsf_gvf + tsf_gvf_finish bit for bit. */
size_t tsf_gvf_one_component_workspace_size(int X, int Y, int Z, int storage);
int tsf_gvf_one_component(const void *d_field4_in, int X, int Y, int Z, float mu, int iterations,
                          int storage, void *d_field4_out, void *d_workspace, size_t workspace_bytes,
                          void *stream);

/* ---------------------------------------------------------------------------
 * Tube detection filter
 * ------------------------------------------------------------------------- */

/* circleFittingTDF (kernels.cl:1065-1157; driver runCircleFittingTDF,
 * tubeDetectionFilters.cpp:57-73): per voxel the Hessian of the field, its
 * eigen-decomposition and the circle-fitting radius sweep
 * r = rmin, rmin+rstep, ... <= rmax with 32 trilinear samples per radius.
 * The Hessian is normalised by w when rmax >= 4.  Writes the response to d_T
 * (float, or uint16 unorm16 when tdf_unorm16 != 0, the reference's 16-bit
 * mode) and the arg-max radius to d_R (float). */
int tsf_tdf_circle(const void *d_field4, int X, int Y, int Z, int storage, float rmin, float rmax,
                   float rstep, void *d_T, int tdf_unorm16, float *d_R, void *stream);

/* tsf_tdf_circle with the kernel forced: mode 1 = one voxel per lane, 2 = one
 * circle sample per lane, 3 = radius sweeps load-balanced within each warp,
 * 0 = the default (2 when every radius is <= 3, else 3).  Identical results. */
int tsf_tdf_circle_mode(const void *d_field4, int X, int Y, int Z, int storage, float rmin,
                        float rmax, float rstep, void *d_T, int tdf_unorm16, float *d_R, int mode,
                        void *stream);

/* Workspace bytes for tsf_tdf_circle_ws: 16 per voxel for the 16-bit storage
 * formats (an x-paired copy of the field), 0 for F32. */
size_t tsf_tdf_workspace_size(int X, int Y, int Z, int storage);

/* tsf_tdf_circle with a workspace (same reference interface, same results bit
 * for bit): for 16-bit storage the call first writes an x-paired copy of the
 * field into the workspace (entry i = texel i and texel i + 1), so that a
 * trilinear sample inside the volume takes four 16-byte loads instead of eight
 * 8-byte ones.  With a smaller or misaligned workspace (16-byte alignment) it
 * behaves as tsf_tdf_circle. */
int tsf_tdf_circle_ws(const void *d_field4, int X, int Y, int Z, int storage, float rmin, float rmax,
                      float rstep, void *d_T, int tdf_unorm16, float *d_R, void *d_workspace,
                      size_t workspace_bytes, void *stream);

/* Options of tsf_tdf_circle_ex.  No counterpart in the reference, whose
 * circleFittingTDF has the sample count and the eigensolver built in. */
typedef struct {
    int samples;   /* circle samples per radius: 32 (the reference, kernels.cl:1122)
                      or another multiple of 4 in [4, 32]                         */
    int stride;    /* sample j takes entry j * stride of the reference's 32-entry
                      cos / sin table (angle j * stride radians), as its disabled
                      sample-count switch does (kernels.cl:1120-1131);
                      (samples - 1) * stride < 32; 1 for the reference           */
    int eigen;     /* 0: tred2 + tql2, the reference's (kernels.cl:1519-1773),
                      bit-exact with it; 1: a closed-form solver in registers (the
                      trigonometric method with Newton steps for the isolated
                      root, robust eigenvectors, an FP64 branch when two
                      eigenvalues nearly coincide); eigenvector signs are
                      canonical (largest component positive), so T and R agree
                      with mode 0 to the circle's sampling noise, not bit for bit */
    int kernel;    /* 0: default (one circle sample per lane for snorm16
                      fields, else the load-balanced sweeps), 1: one voxel per
                      lane, 2: one circle sample per lane (a warp evaluates one
                      voxel-radius at a time), 3: load-balanced sweeps; all give
                      the same bits                                             */
} tsf_tdf_options;

/* tsf_tdf_circle_ws with options (NULL: the reference's 32 samples, tql2,
 * default kernel -- then identical to tsf_tdf_circle_ws). */
int tsf_tdf_circle_ex(const void *d_field4, int X, int Y, int Z, int storage, float rmin, float rmax,
                      float rstep, const tsf_tdf_options *options, void *d_T, int tdf_unorm16, float *d_R,
                      void *d_workspace, size_t workspace_bytes, void *stream);

/* splineTDF (kernels.cl:1159-1254, kernels_no_3d_write.cl:1574-1671; driver
 * runSplineTDF, tubeDetectionFilters.cpp:4-55, called with
 * max(1.5, radius-min) at tube-segmentation.cpp:785-786): the normalised
 * Hessian's eigenvectors, then 12 arms in the plane of e2 and e3, each a line
 * search from max(1, rmin) in steps of rstep up to rmax for the first border
 * point of the field magnitude (minimum mean rise 0.1).  T = 0 where an arm
 * finds none or the border field points along the arm, else
 * min(1, mean(1 - |n . e1|) * symmetry + 0.2); R = the sum of the radii found
 * / 12.  T as float, or unorm16 when tdf_unorm16 != 0.  At most 4096 radii per
 * arm (the reference does not end the search for a step that does not
 * advance the radius). */
int tsf_tdf_spline(const void *d_field4, int X, int Y, int Z, int storage, float rmin, float rmax,
                   float rstep, void *d_T, int tdf_unorm16, float *d_R, void *stream);

/* combine (kernels.cl:561-572, tube-segmentation.cpp:802-824): where the small
 * TDF exceeds the large one, take it and its radius.  d_T_large / d_R_large
 * are updated in place; T arrays are float or unorm16 per tdf_unorm16. */
int tsf_tdf_combine(const void *d_T_small, const float *d_R_small, void *d_T_large,
                    float *d_R_large, int64_t n, int tdf_unorm16, void *stream);

/* ---------------------------------------------------------------------------
 * Centerline linking
 * ------------------------------------------------------------------------- */

/* runNewCenterlineAlg after the vertex list (parallelCenterlineExtraction.cpp:
 * 911-1161; kernels linkLengths, compact, linkCenterpoints,
 * removeDuplicateEdges, graphComponentLabeling, calculateTreeLength,
 * kernels.cl:327-508, and the 2-D pyramid enumeration of the edge image).
 * d_vertices: n_vertices x 3 int (x, y, z), n_vertices <= 16384; d_T: the TDF
 * (float, or unorm16 when tdf_unorm16 != 0).  Writes the edges (pairs of
 * vertex indices, at most 2 n_vertices, in the reference's pyramid order) to
 * d_edges and their count to *n_edges (host; the call synchronises
 * `stream`), each vertex's component label (the smallest vertex index of the
 * component) to d_labels and the component sizes, indexed by label, to
 * d_tree_sizes.  Candidate partners are listed in ascending index (the
 * reference's atomic compaction leaves that order, and so the choice between
 * pairs of equal length, to chance).  TSF_ERR_COUNT_RANGE ("No edges were
 * found") when nothing links. */
size_t tsf_link_workspace_size(int n_vertices);
int tsf_link_centerpoints(const int *d_vertices, int n_vertices, const void *d_T, int tdf_unorm16,
                          int X, int Y, int Z, float min_mean_tdf, float max_distance, int *d_edges,
                          int *n_edges, int *d_labels, int *d_tree_sizes, void *d_workspace,
                          size_t workspace_bytes, void *stream);

/* removeSmallTrees (kernels.cl:510-534; the reference's GPU rasterisation,
 * used when loop removal is off): sets d_centerlines (X*Y*Z int8, zeroed by
 * the caller) to 1 along the edges of components of at least
 * min_tree_length vertices. */
int tsf_rasterize_trees(const int *d_vertices, const int *d_edges, int n_edges, const int *d_labels,
                        const int *d_tree_sizes, int min_tree_length, int8_t *d_centerlines, int X,
                        int Y, int Z, void *stream);

/* Host functions (no device memory): the CPU part of runNewCenterlineAlg
 * when loop removal or a VTK centerline file is requested
 * (parallelCenterlineExtraction.cpp:1168-1247).
 *
 * tsf_centerline_graph: from the linked graph (vertices, edges, labels and
 * tree sizes as tsf_link_centerpoints gives them, copied to the host) keeps
 * the trees of at least min_tree_length vertices, splits edges longer than
 * max_edge_distance (0 = no splitting; the reference splits only for the VTK
 * file), removes loops (removeLoops, :129-285) and rasterises the result
 * into centerlines (X*Y*Z int8, written) while replacing the radius along
 * each edge by its mean (createCenterlineVoxels, :287-321; radius X*Y*Z
 * float, updated).  The final graph goes to out_vertices (x, y, z) and
 * out_edges; both counts are returned, and TSF_ERR_CAPACITY when either
 * exceeds `capacity` (radius and centerlines are then left unchanged: call
 * again with more).  TSF_ERR_COUNT_RANGE when no
 * vertex survives ("Centerline graph size is 0").
 * tsf_remove_loops: removeLoops alone.
 * tsf_write_centerline_vtk: writeToVtkFile (inputOutput.cpp:48-63). */
int tsf_centerline_graph(const int *vertices, int n_vertices, const int *edges, int n_edges,
                         const int *labels, const int *tree_sizes, int min_tree_length,
                         int max_edge_distance, int X, int Y, int Z, float *radius,
                         int8_t *centerlines, int *out_vertices, int *out_edges, int capacity,
                         int *n_out_vertices, int *n_out_edges);
/* tsf_centerline_graph for volumes kept on the device: the same graph
 * (out_vertices, out_edges, both counts, the capacity rule) and, instead of
 * writing centerlines and radius, the cells createCenterlineVoxels visits
 * (parallelCenterlineExtraction.cpp:287-321), edge after edge in order:
 * cells[edge_start[k] .. edge_start[k+1]) for output edge k, as x + X*(y +
 * Y*z); edge_start holds n_out_edges + 1 entries (room for capacity + 1).
 * *n_cells is returned too, and TSF_ERR_CAPACITY also when it exceeds
 * cell_capacity.
 * tsf_centerline_smooth_radius: given values[i] = radius at cells[i] (read
 * with tsf_gather_cells), replays the edge-ordered mean of the radius along
 * each edge and returns each distinct cell once, in first-visit order, with
 * its final radius (room for edge_start[n_edges] entries).
 * tsf_gather_cells / tsf_centerline_apply (device): d_values[i] =
 * d_volume[d_cells[i]]; d_centerlines[d_cells[i]] = 1 and, unless d_radius
 * is NULL, d_radius[d_cells[i]] = d_values[i].  Cells outside [0, X*Y*Z)
 * are skipped.  Together these give the centerlines and radius of
 * tsf_centerline_graph without copying the volumes to the host. */
int tsf_centerline_graph_cells(const int *vertices, int n_vertices, const int *edges, int n_edges,
                               const int *labels, const int *tree_sizes, int min_tree_length,
                               int max_edge_distance, int X, int Y, int Z, int *out_vertices,
                               int *out_edges, int capacity, int *n_out_vertices, int *n_out_edges,
                               int64_t *cells, int64_t *edge_start, int64_t cell_capacity,
                               int64_t *n_cells);
int tsf_centerline_smooth_radius(const int64_t *cells, const int64_t *edge_start, int n_edges,
                                 const float *values, int64_t *unique_cells, float *unique_values,
                                 int64_t *n_unique);
int tsf_gather_cells(const float *d_volume, int X, int Y, int Z, const int64_t *d_cells,
                     int64_t n_cells, float *d_values, void *stream);
int tsf_centerline_apply(int8_t *d_centerlines, float *d_radius, int X, int Y, int Z,
                         const int64_t *d_cells, const float *d_values, int64_t n_cells,
                         void *stream);
int tsf_remove_loops(const int *vertices, int n_vertices, const int *edges, int n_edges, int X,
                     int Y, int Z, int *out_vertices, int *out_edges, int capacity,
                     int *n_out_vertices, int *n_out_edges);
int tsf_write_centerline_vtk(const char *path, const int *vertices, int n_vertices,
                             const int *edges, int n_edges);

/* ---------------------------------------------------------------------------
 * Cropping (the input stage)
 * ------------------------------------------------------------------------- */

/* Workspace bytes for tsf_crop_scan_lines. */
size_t tsf_crop_workspace_size(int X, int Y, int Z);

/* cropDatasetThreshold (method 0) / cropDatasetLung (method 1),
 * kernels.cl:813-946, enqueued for the three slice directions at
 * tube-segmentation.cpp:1577-1604: d_volume is the raw volume of TSF_TYPE_*
 * `type` (before toFloat); d_counts (X + Y + Z int16: slices along x, then y,
 * then z) receives, per slice, the number of scan lines that are inside --
 * with a voxel above `threshold` (method 0), or whose HU run-length state
 * machine (limit -150, +1024 for unsigned data; runs of 30) finds two white
 * areas and one black or more than one of each (method 1; integer data only). */
int tsf_crop_scan_lines(const void *d_volume, int type, int X, int Y, int Z, int method, float threshold,
                        int16_t *d_counts, void *d_workspace, size_t workspace_bytes, void *stream);

/* Host (no device memory): the crop box from the counts
 * (tube-segmentation.cpp:1611-1719).  box receives x1, y1, z1 and the cropped
 * extents SX, SY, SZ (multiples of 4 where the volume allows, as the reference
 * rounds them).  start_z_middle: the z search of "cropping-start-z middle"
 * (used by the lung cropping) instead of "end".  TSF_ERR_INVALID_ARG ("Invalid
 * cropping to new size ...") for an empty box. */
int tsf_crop_bounds(const int16_t *counts, int X, int Y, int Z, int min_scan_lines, int start_z_middle, int *box);

/* Host: the fixed in-plane crop of the AAA-Vessels-CT preset without cropping
 * (tube-segmentation.cpp:1747-1772): round(extent * fraction) removed from both
 * sides of x and y, every extent then shrunk to a multiple of 4.  box as above. */
int tsf_crop_box_fixed(int X, int Y, int Z, float fraction, int *box);

/* Copies box (x1, y1, z1, SX, SY, SZ) of the raw volume to d_out (SX*SY*SZ
 * elements of `type`, x fastest) -- the reference's enqueueCopyImage of the
 * cropped region (tube-segmentation.cpp:1727-1744). */
int tsf_crop_copy(const void *d_volume, int type, int X, int Y, int Z, const int *box, void *d_out, void *stream);

/* ---------------------------------------------------------------------------
 * Segmentation
 * ------------------------------------------------------------------------- */

/* Workspace bytes for tsf_segment_inverse_gradient. */
size_t tsf_segment_workspace_size(int X, int Y, int Z);

/* runInverseGradientSegmentation (segmentation.cpp:5-205; kernels
 * initGrowing, grow, dilate, erode, kernels_no_3d_write.cl:1100-1207 and
 * 1370-1412).  d_centerlines: X*Y*Z int8 (1 on the centerline); d_field4: the
 * vector field the TDF was computed on (vx, vy, vz, |v|) in `storage`;
 * d_radius: X*Y*Z float.  Grows from the centerline against the field
 * magnitude until an iteration accepts nothing, then closes the result
 * (3x3x3 dilation, then erosion) into d_segmentation (X*Y*Z int8, 0 / 1,
 * every voxel written).  Within one grow iteration the reference's writes race
 * (a voxel's own verdict against its neighbours' "check it" marks); here the
 * iteration decides first and applies second, with the precedence accepted >
 * to check > dropped.  *iterations (may be null) receives the number of grow
 * iterations, the last of which accepted nothing.  Synchronises `stream`. */
int tsf_segment_inverse_gradient(const int8_t *d_centerlines, const void *d_field4, int storage,
                                 const float *d_radius, int X, int Y, int Z, int8_t *d_segmentation,
                                 int *iterations, void *d_workspace, size_t workspace_bytes,
                                 void *stream);

/* runSphereSegmentation (segmentation.cpp:207-307; kernel
 * sphereSegmentation, kernels_no_3d_write.cl:1209-1234): d_segmentation
 * (X*Y*Z int8, written) is 1 within distance < radius of every voxel with
 * d_centerlines != 0. */
int tsf_segment_spheres(const int8_t *d_centerlines, const float *d_radius, int X, int Y, int Z,
                        int8_t *d_segmentation, void *stream);

/* Reverse-mode derivative of tsf_tdf_circle (no counterpart in the
 * reference): given d_gT = dL/dT (float per voxel), ADDS dL/d(field x,y,z) to
 * d_gfield (planar FP32, 3N) -- through the trilinear samples at the arg-max
 * radius, through the sample directions (eigenvectors of the Hessian, by
 * first-order eigenvector perturbation) and through the Hessian's central
 * differences (of v/|v| when rmax >= 4, w taken as |v|).  The arg-max radius
 * is held fixed (sub-gradient of the max over radii).  d_T, d_R: the float
 * response and radius tsf_tdf_circle wrote for this field and radius range
 * (then the sweep is not repeated), or both NULL (the sweep is recomputed).
 * Scatters use atomics, so the last bits vary between runs. */
size_t tsf_tdf_backward_workspace_size(int X, int Y, int Z);
int tsf_tdf_circle_backward(const void *d_field4, int X, int Y, int Z, int storage, float rmin,
                            float rmax, float rstep, const float *d_gT, const float *d_T,
                            const float *d_R, float *d_gfield, void *d_workspace,
                            size_t workspace_bytes, void *stream);

/* Reverse-mode derivative of tsf_vector_field with respect to its input
 * volume: ADDS to d_gin the gradient from d_gf (planar FP32 dL/df). */
int tsf_vector_field_backward(const float *d_in, const float *d_gf, int X, int Y, int Z, float fmax,
                              int vsign, float *d_gin, void *stream);

/* Reverse-mode derivative of tsf_blur: ADDS the transposed blur of d_gout to
 * d_gin and, when dsigma is not NULL, writes dL/dsigma (host, FP64; the call
 * then synchronises `stream`). */
size_t tsf_blur_backward_workspace_size(int X, int Y, int Z);
int tsf_blur_backward(const float *d_in, const float *d_gout, int X, int Y, int Z, float sigma,
                      float *d_gin, double *dsigma, void *d_workspace, size_t workspace_bytes,
                      void *stream);

/* ---------------------------------------------------------------------------
 * Candidate centerpoints
 * ------------------------------------------------------------------------- */

/* Workspace bytes for tsf_candidates. */
size_t tsf_candidates_workspace_size(int X, int Y, int Z);

/* The front half of runNewCenterlineAlg (parallelCenterlineExtraction.cpp:
 * 667-899): threshold (findCandidateCenterpoints, kernels.cl:1296-1307),
 * compaction in histogram-pyramid order (kernels.cl:63-299, oul
 * HistogramPyramid3D), the cross-section non-maximum filter
 * (findCandidateCenterpoints2, kernels.cl:1309-1390), the per-cube arg-max
 * (dd, kernels.cl:1260-1292) and a second compaction into the vertex list.
 *
 *  d_T          TDF (float or unorm16 per tdf_unorm16); d_R radius (float);
 *  d_field4     the GVF result image (w = |v|);
 *  d_vertices   int32 (x,y,z) triples, capacity max_vertices, written in the
 *               pyramid's order (x, z, y bit-interleaved key);
 *  d_centerpoints  optional (may be NULL) int8 volume receiving the filtered
 *               candidate mask (the reference's `centerpoints-only` output);
 *  d_candidates optional (may be NULL) int32 triples receiving the candidate
 *               list before filtering, capacity max_candidates;
 *  n_candidates, n_vertices  host outputs.
 * Synchronises `stream` twice (the counts are needed on the host, as the
 * reference's getSum() calls are).  Returns TSF_ERR_COUNT_RANGE, with the
 * counts still written, when the candidate count is not in (0, N/2] or the
 * vertex count is not in [8, 16384), the reference's sanity checks. */
int tsf_candidates(const void *d_T, int tdf_unorm16, const float *d_R, const void *d_field4,
                   int storage, int X, int Y, int Z, float tdf_high, int cube_size,
                   int32_t *d_vertices, int64_t max_vertices, int8_t *d_centerpoints,
                   int32_t *d_candidates, int64_t max_candidates, int64_t *n_candidates,
                   int64_t *n_vertices, void *d_workspace, size_t workspace_bytes, void *stream);

/* Workspace bytes for tsf_compact_mask. */
size_t tsf_compact_workspace_size(int X, int Y, int Z);

/* The histogram-pyramid enumeration alone (createPositions3D,
 * kernels.cl:279-299): positions of the voxels with d_mask[i] != 0, ordered
 * by the pyramid traversal.  Synchronises `stream`. */
int tsf_compact_mask(const int8_t *d_mask, int X, int Y, int Z, int32_t *d_positions,
                     int64_t max_positions, int64_t *count, void *d_workspace,
                     size_t workspace_bytes, void *stream);

/* ---------------------------------------------------------------------------
 * Multigrid GVF
 * ------------------------------------------------------------------------- */

/* Workspace bytes for tsf_gvf_fmg. */
size_t tsf_gvf_fmg_workspace_size(int X, int Y, int Z, int storage);

/* runFMGGVF (gradientVectorFlow.cpp:729-1005; kernels.cl:1775-2061): full
 * multigrid with v0 = 1, v1 = 2, v2 = 2, three levels, `iterations` FMG cycles
 * per component.  d_field4_in is the vector field image (createVectorField
 * output); d_field4_out receives (vx, vy, vz, |v|).  All intermediate images
 * are rounded to `storage`. */
int tsf_gvf_fmg(const void *d_field4_in, void *d_field4_out, int X, int Y, int Z, float mu,
                int iterations, int storage, void *d_workspace, size_t workspace_bytes,
                void *stream);

#ifdef __cplusplus
}
#endif
#endif /* TSF_C_H */
