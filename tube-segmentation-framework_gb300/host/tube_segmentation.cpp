// tube_segmentation.cpp -- run() / runSegmentation(): the reference's library
// entry point (tube-segmentation.cpp:53-163) driving the GPU hot path through
// the C ABI of this library.
//
// Stage order and parameter semantics follow the reference:
//  readDatasetAndTransfer  (tube-segmentation.cpp:1399-1905): .mhd header,
//      raw data, limits (getLimits :1380-1396), upload, then lung or
//      threshold cropping, the AAA-Vessels-CT in-plane crop or the shrink to
//      a multiple of 4 on the device, toFloat;
//  runCircleFittingMethod  (:212-939): small-radius TDF on the un-diffused
//      field when radius-min < 2.5, GVF (Jacobi or FMG) of the large-blur
//      field, large-radius TDF, combine;
//  runNewCenterlineAlg (parallelCenterlineExtraction.cpp:667-1332): candidate
//      centerpoints and vertices, linking into trees (GPU), then either the
//      host loop removal and rasterisation (loop-removal or a VTK file) or
//      the GPU rasterisation of the large trees;
//  runInverseGradientSegmentation / runSphereSegmentation (segmentation.cpp):
//      unless no-segmentation, on the centerlines, the GVF field and the
//      radius (averaged along the edges after host loop removal).
// The reference's GVF loop returns the result of iterations - 1 when the
// iteration count is odd (gradientVectorFlow.cpp:1137-1172); run() does the
// same.  Options outside this library's scope (other centerline methods, a
// CPU device) raise SIPL::SIPLException.  With use-spline-tdf the large-radius
// TDF is the spline TDF (from max(1.5, radius-min), tube-segmentation.cpp:785-789).
#include <cuda_runtime_api.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <limits>
#include <memory>
#include <sstream>
#include <vector>

#include <fcntl.h>
#include <unistd.h>

#include "first_touch.hpp"
#include "tsf/tsf_c.h"
#include "tsf/tube-segmentation.hpp"

namespace {

[[noreturn]] void raise(const std::string &msg) { throw SIPL::SIPLException(msg.c_str()); }

void check(int code, const char *what) {
    if (code == TSF_OK) return;
    raise(std::string(what) + ": " + tsf_last_error_string());
}

void check_cuda(cudaError_t e, const char *what) {
    if (e != cudaSuccess) raise(std::string(what) + ": " + cudaGetErrorString(e));
}

// Device buffer owned by a scope unless released.
struct DevBuf {
    void *p = nullptr;
    DevBuf() = default;
    explicit DevBuf(size_t bytes) { alloc(bytes); }
    void alloc(size_t bytes) {
        if (p) cudaFree(p);
        p = nullptr;
        check_cuda(cudaMalloc(&p, bytes ? bytes : 256), "cudaMalloc");
    }
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    void *release() {
        void *q = p;
        p = nullptr;
        return q;
    }
    template <typename T> T *as() const { return reinterpret_cast<T *>(p); }
    void swap(DevBuf &o) { std::swap(p, o.p); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
};

struct Stream {
    cudaStream_t s = nullptr;
    Stream() { check_cuda(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate"); }
    ~Stream() {
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    }
};

// The "timing" parameter (parameters:21): each stage's duration printed as
// "RUNTIME <stage>: <ms> ms", as the reference does with a marker before and
// after the stage and a finish of its queue at the second one
// (tube-segmentation.cpp:297-298,446-452 and the other stages).  Here the
// markers are events on the run's stream, so a stage's time includes host
// work between its launches; host-only stages use the host clock.  Off: no
// events, no synchronisation.
class StageTimer {
  public:
    StageTimer(bool on, cudaStream_t s) : on_(on), s_(s) {
        if (!on_) return;
        check_cuda(cudaEventCreate(&e0_), "cudaEventCreate");
        check_cuda(cudaEventCreate(&e1_), "cudaEventCreate");
    }
    ~StageTimer() {
        if (e0_) cudaEventDestroy(e0_);
        if (e1_) cudaEventDestroy(e1_);
    }
    bool on() const { return on_; }
    void start() {
        if (on_) check_cuda(cudaEventRecord(e0_, s_), "cudaEventRecord");
    }
    void stop(const char *stage) {
        if (!on_) return;
        check_cuda(cudaEventRecord(e1_, s_), "cudaEventRecord");
        check_cuda(cudaEventSynchronize(e1_), "cudaEventSynchronize");
        float ms = 0.0f;
        check_cuda(cudaEventElapsedTime(&ms, e0_, e1_), "cudaEventElapsedTime");
        std::cout << "RUNTIME " << stage << ": " << ms << " ms" << std::endl;
    }
    void host_start() { h0_ = std::chrono::steady_clock::now(); }
    void host_stop(const char *stage) {
        if (!on_) return;
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - h0_).count();
        std::cout << "RUNTIME " << stage << ": " << ms << " ms" << std::endl;
    }
    StageTimer(const StageTimer &) = delete;
    StageTimer &operator=(const StageTimer &) = delete;

  private:
    bool on_;
    cudaStream_t s_;
    cudaEvent_t e0_ = nullptr, e1_ = nullptr;
    std::chrono::steady_clock::time_point h0_;
};

std::string trim(const std::string &v) {
    size_t b = 0, e = v.size();
    while (b < e && std::isspace((unsigned char)v[b])) b++;
    while (e > b && std::isspace((unsigned char)v[e - 1])) e--;
    return v.substr(b, e - b);
}

// value of "Key = value" lines; empty if the line is another key
bool header_value(const std::string &line, const char *key, std::string &value) {
    const size_t k = std::strlen(key);
    if (line.compare(0, k, key) != 0) return false;
    const size_t eq = line.find('=', k);
    if (eq == std::string::npos) return false;
    value = trim(line.substr(eq + 1));
    return true;
}

struct HostVolume {
    std::unique_ptr<char[]> data;   // the raw file, not initialised before the read
    size_t bytes = 0;
    int type = -1;           // TSF_TYPE_*
    int elem = 0;
    SIPL::int3 size;
    SIPL::float3 spacing{1, 1, 1};
};

// Minimum and maximum of p[0, n) as the reference's getMinimum/getMaximum
// fold them (tube-segmentation.cpp:1380-1396): from numeric_limits<T>::max()
// and ::min(), std::min / std::max per element.
template <typename T> struct Limits {
    T mn = std::numeric_limits<T>::max(), mx = std::numeric_limits<T>::min();
    void fold(const T *p, size_t n) {
        for (size_t i = 0; i < n; i++) {
            mn = std::min(mn, p[i]);
            mx = std::max(mx, p[i]);
        }
    }
};

// Reads `bytes` of the file at fd into dst with up to 16 threads, each one
// contiguous slice (pread), and folds each slice into its own Limits<T> while
// it is still in cache when `limits` is set.  The slices' results are folded
// in file order: std::min / std::max keep the first of equal values and never
// take a NaN, so the result equals the sequential fold over the whole file.
template <typename T>
bool read_slices(int fd, char *dst, size_t bytes, bool limits, float &lo, float &hi) {
    const size_t nt = tsf_host::host_threads(bytes);
    const size_t elems = bytes / sizeof(T), per = (elems + nt - 1) / nt;
    std::vector<Limits<T>> part(nt);
    std::vector<char> ok(nt, 0);
    auto work = [&](size_t t) {
        const size_t e0 = std::min(elems, t * per), e1 = std::min(elems, e0 + per);
        size_t off = e0 * sizeof(T);
        const size_t end = t + 1 == nt ? bytes : e1 * sizeof(T);
        while (off < end) {
            const ssize_t r = pread(fd, dst + off, end - off, (off_t)off);
            if (r <= 0) return;
            off += (size_t)r;
        }
        if (limits) part[t].fold(reinterpret_cast<const T *>(dst) + e0, e1 - e0);
        ok[t] = 1;
    };
    tsf_host::parallel_tasks(nt, work);
    Limits<T> all;
    for (size_t t = 0; t < nt; t++) {
        if (!ok[t]) return false;
        all.mn = std::min(all.mn, part[t].mn);
        all.mx = std::max(all.mx, part[t].mx);
    }
    lo = (float)all.mn;
    hi = (float)all.mx;
    return true;
}

HostVolume read_volume(const std::string &filename, paramList &parameters, float &minimum, float &maximum) {
    std::ifstream mhd(filename.c_str());
    if (!mhd) throw SIPL::IOException(filename.c_str(), __LINE__, __FILE__);
    HostVolume v;
    std::string line, value, typeName, rawName;
    bool haveSize = false;
    while (std::getline(mhd, line)) {
        if (header_value(line, "ElementType", value)) {
            std::istringstream(value) >> typeName;
        } else if (header_value(line, "ElementDataFile", value)) {
            std::istringstream(value) >> rawName;
        } else if (header_value(line, "DimSize", value)) {
            std::istringstream in(value);
            in >> v.size.x >> v.size.y >> v.size.z;
            haveSize = (bool)in;
        } else if (header_value(line, "ElementSpacing", value)) {
            std::istringstream in(value);
            in >> v.spacing.x >> v.spacing.y >> v.spacing.z;
        }
    }
    if (typeName.empty() || rawName.empty() || !haveSize)
        throw SIPL::SIPLException("Error reading mhd file. Type, filename or size not found", __LINE__, __FILE__);
    const size_t slash = filename.rfind('/');
    if (slash != std::string::npos) rawName = filename.substr(0, slash + 1) + rawName;

    if (typeName == "MET_SHORT") { v.type = TSF_TYPE_INT16; v.elem = 2; }
    else if (typeName == "MET_USHORT") { v.type = TSF_TYPE_UINT16; v.elem = 2; }
    else if (typeName == "MET_CHAR") { v.type = TSF_TYPE_INT8; v.elem = 1; }
    else if (typeName == "MET_UCHAR") { v.type = TSF_TYPE_UINT8; v.elem = 1; }
    else if (typeName == "MET_FLOAT") { v.type = TSF_TYPE_FLOAT32; v.elem = 4; }
    else raise("unsupported data type " + typeName);

    const size_t bytes = (size_t)v.size.x * v.size.y * v.size.z * v.elem;
    v.data.reset(new char[bytes ? bytes : 1]);
    v.bytes = bytes;
    struct File {
        int fd;
        ~File() {
            if (fd >= 0) close(fd);
        }
    } file{open(rawName.c_str(), O_RDONLY)};
    const int fd = file.fd;
    if (fd < 0) throw SIPL::IOException(rawName.c_str(), __LINE__, __FILE__);
    // getLimits (tube-segmentation.cpp:1380-1396); its result is used only
    // where "minimum" or "maximum" is off
    const std::string pmin = getParamStr(parameters, "minimum"), pmax = getParamStr(parameters, "maximum");
    const bool limits = pmin == "off" || pmax == "off";
    float lo = 0.0f, hi = 1.0f;
    bool got = false;
    switch (v.type) {
    case TSF_TYPE_INT16: got = read_slices<int16_t>(fd, v.data.get(), bytes, limits, lo, hi); break;
    case TSF_TYPE_UINT16: got = read_slices<uint16_t>(fd, v.data.get(), bytes, limits, lo, hi); break;
    case TSF_TYPE_INT8: got = read_slices<int8_t>(fd, v.data.get(), bytes, limits, lo, hi); break;
    case TSF_TYPE_UINT8: got = read_slices<uint8_t>(fd, v.data.get(), bytes, limits, lo, hi); break;
    default: got = read_slices<float>(fd, v.data.get(), bytes, limits, lo, hi); break;
    }
    if (!got) throw SIPL::IOException(rawName.c_str(), __LINE__, __FILE__);
    minimum = pmin != "off" ? (float)std::atof(pmin.c_str()) : lo;
    maximum = pmax != "off" ? (float)std::atof(pmax.c_str()) : hi;
    if (v.type == TSF_TYPE_UINT16) {
        // unsigned CT data with the airway / AAA presets: HU limits shifted by 1024
        const std::string preset = getParamStr(parameters, "parameters");
        if (preset == "Lung-Airways-CT" || preset == "AAA-Vessels-CT") {
            minimum = (float)std::atof(pmin.c_str()) + 1024.0f;
            maximum = (float)std::atof(pmax.c_str()) + 1024.0f;
        }
    }
    return v;
}

// readDatasetAndTransfer after the upload (tube-segmentation.cpp:1556-1828):
// lung or threshold cropping (scan-line counts on the GPU, the box on the
// host), else the fixed in-plane crop of the AAA-Vessels-CT preset, else the
// shrink of every extent to a multiple of 4.  box = x1, y1, z1, SX, SY, SZ;
// returns the shift vector (left at zero by the AAA crop, as in the reference).
SIPL::int3 input_box(paramList &P, const HostVolume &hv, const void *d_raw, cudaStream_t s, int *box) {
    const int X = hv.size.x, Y = hv.size.y, Z = hv.size.z;
    const std::string cropping = getParamStr(P, "cropping");
    if (cropping == "lung" || cropping == "threshold") {
        std::cout << "performing cropping" << std::endl;
        const bool lung = cropping == "lung";
        const int min_lines = (int)getParam(P, lung ? "min-scan-lines-lung" : "min-scan-lines-threshold");
        const bool middle = lung || getParamStr(P, "cropping-start-z") == "middle";
        const size_t wsb = tsf_crop_workspace_size(X, Y, Z);
        DevBuf ws(wsb), counts(sizeof(int16_t) * ((size_t)X + Y + Z));
        check(tsf_crop_scan_lines(d_raw, hv.type, X, Y, Z, lung ? 1 : 0, lung ? 0.0f : getParam(P, "cropping-threshold"),
                                  counts.as<int16_t>(), ws.p, wsb, (void *)s),
              "cropping");
        std::vector<int16_t> hc((size_t)X + Y + Z);
        check_cuda(cudaMemcpyAsync(hc.data(), counts.p, hc.size() * sizeof(int16_t), cudaMemcpyDeviceToHost, s),
                   "cropping");
        check_cuda(cudaStreamSynchronize(s), "cropping");
        if (tsf_crop_bounds(hc.data(), X, Y, Z, min_lines, middle ? 1 : 0, box) != TSF_OK)
            raise(tsf_last_error_string());
        std::cout << "Dataset cropped to " << box[3] << ", " << box[4] << ", " << box[5] << std::endl;
        return SIPL::int3(box[0], box[1], box[2]);
    }
    if (getParamStr(P, "parameters") == "AAA-Vessels-CT") {
        check(tsf_crop_box_fixed(X, Y, Z, 0.15f, box), "cropping");
        std::cout << "NOTE: reduced size to " << box[3] << ", " << box[4] << ", " << box[5] << std::endl;
        return SIPL::int3(0, 0, 0);
    }
    box[0] = box[1] = box[2] = 0;
    box[3] = X - X % 4;
    box[4] = Y - Y % 4;
    box[5] = Z - Z % 4;
    if (box[3] != X || box[4] != Y || box[5] != Z)
        std::cout << "NOTE: reduced size to " << box[3] << ", " << box[4] << ", " << box[5] << std::endl;
    return SIPL::int3(0, 0, 0);
}

int storage_from_parameters(paramList &p) {
    const std::string s = getParamStr(p, "gvf-storage");
    if (s == "f32") return TSF_STORE_F32;
    if (s == "f16") return TSF_STORE_F16;
    if (s == "bf16") return TSF_STORE_BF16;
    if (s == "snorm16") return TSF_STORE_SNORM16;
    return (getParamBool(p, "16bit-vectors") && !getParamBool(p, "32bit-vectors")) ? TSF_STORE_SNORM16
                                                                                    : TSF_STORE_F32;
}

struct FieldResult {
    DevBuf T, R, field;
};

// runCircleFittingMethod, tube-segmentation.cpp:212-939
void circle_fitting_method(paramList &P, const float *d_vol, int X, int Y, int Z, int st, bool tdf16,
                           cudaStream_t s, StageTimer &tm, FieldResult &out) {
    const float rMin = getParam(P, "radius-min"), rMax = getParam(P, "radius-max"), rStep = getParam(P, "radius-step");
    const float fmax = getParam(P, "fmax");
    const int vsign = getParamStr(P, "mode") == "black" ? -1 : 1;
    const float smallBlur = getParam(P, "small-blur"), largeBlur = getParam(P, "large-blur");
    const size_t n = (size_t)X * Y * Z, es = tsf_storage_bytes(st), ts = tdf16 ? 2 : 4;
    void *S = (void *)s;

    DevBuf Ts, Rs, f4small;
    if (rMin < 2.5f) {
        tm.start();
        DevBuf blurred;
        const float *src = d_vol;
        if (smallBlur > 0) {
            blurred.alloc(n * 4);
            check(tsf_blur(d_vol, blurred.as<float>(), X, Y, Z, smallBlur, S), "blur");
            src = blurred.as<float>();
        }
        f4small.alloc(n * 4 * es);
        check(tsf_vector_field(src, X, Y, Z, fmax, vsign, st, nullptr, f4small.p, S), "vector field");
        tm.stop("of Create vector field");
        tm.start();
        Ts.alloc(n * ts);
        Rs.alloc(n * 4);
        const size_t twb = tsf_tdf_workspace_size(X, Y, Z, st);
        DevBuf tws(twb);
        check(tsf_tdf_circle_ws(f4small.p, X, Y, Z, st, rMin, 3.0f, 0.5f, Ts.p, tdf16, Rs.as<float>(), tws.p, twb, S),
              "TDF");
        tm.stop("of TDF small");
        if (rMax < 2.5f) {
            out.T.p = Ts.release();
            out.R.p = Rs.release();
            out.field.p = f4small.release();
            return;
        }
        f4small.alloc(0);   // free early, as the reference does
    }

    tm.start();
    DevBuf blurred;
    const float *src = d_vol;
    if (largeBlur > 0) {
        blurred.alloc(n * 4);
        check(tsf_blur(d_vol, blurred.as<float>(), X, Y, Z, largeBlur, S), "blur");
        src = blurred.as<float>();
    }
    tm.stop("blurring");
    out.field.alloc(n * 4 * es);
    const int iterations = (int)getParam(P, "gvf-iterations");
    const float mu = getParam(P, "gvf-mu");
    if (getParamBool(P, "use-fmg-gvf")) {
        tm.start();
        DevBuf f4in(n * 4 * es);
        check(tsf_vector_field(src, X, Y, Z, fmax, vsign, st, nullptr, f4in.p, S), "vector field");
        blurred.alloc(0);
        tm.stop("Create vector field");
        tm.start();
        DevBuf ws(tsf_gvf_fmg_workspace_size(X, Y, Z, st));
        check(tsf_gvf_fmg(f4in.p, out.field.p, X, Y, Z, mu, iterations, st, ws.p,
                          tsf_gvf_fmg_workspace_size(X, Y, Z, st), S), "multigrid GVF");
        tm.stop("of GVF");
    } else {
        tm.start();
        DevBuf f0(n * 3 * es), v(n * 3 * es);
        check(tsf_vector_field(src, X, Y, Z, fmax, vsign, st, f0.p, nullptr, S), "vector field");
        blurred.alloc(0);
        tm.stop("Create vector field");
        tm.start();
        check_cuda(cudaMemcpyAsync(v.p, f0.p, n * 3 * es, cudaMemcpyDeviceToDevice, s), "copy");
        const size_t wsb = tsf_gvf_workspace_size(X, Y, Z, st);
        DevBuf ws(wsb);
        // the reference's ping-pong returns the even part of the iteration count
        check(tsf_gvf(f0.p, v.p, X, Y, Z, mu, iterations - iterations % 2, st, ws.p, wsb, S), "GVF");
        check(tsf_gvf_finish(v.p, out.field.p, X, Y, Z, st, S), "GVF finish");
        tm.stop("of GVF");
    }
    tm.start();
    out.T.alloc(n * ts);
    out.R.alloc(n * 4);
    if (getParamBool(P, "use-spline-tdf"))
        check(tsf_tdf_spline(out.field.p, X, Y, Z, st, std::max(1.5f, rMin), rMax, rStep, out.T.p, tdf16,
                             out.R.as<float>(), S), "spline TDF");
    else {
        const size_t twb = tsf_tdf_workspace_size(X, Y, Z, st);
        DevBuf tws(twb);
        check(tsf_tdf_circle_ws(out.field.p, X, Y, Z, st, std::max(2.5f, rMin), rMax, rStep, out.T.p, tdf16,
                                out.R.as<float>(), tws.p, twb, S),
              "TDF");
    }
    tm.stop("of TDF large");
    if (rMin < 2.5f) {
        tm.start();
        check(tsf_tdf_combine(Ts.p, Rs.as<float>(), out.T.p, out.R.as<float>(), (int64_t)n, tdf16, S), "combine");
        tm.stop("of combine");
    }
}

}  // namespace

TSFOutput *run(std::string filename, paramList &parameters, std::string /*kernel_dir*/) {
    if (getParamStr(parameters, "device") != "gpu")
        raise("device " + getParamStr(parameters, "device") + " is not supported: this library runs on the GPU");
    const std::string method = getParamStr(parameters, "centerline-method");
    if (method != "gpu") raise("centerline-method " + method + " is not part of this library (use gpu)");

    // the file first: a missing file raises SIPL::IOException before any device work
    const bool timing = getParamBool(parameters, "timing");
    float minimum = 0.0f, maximum = 1.0f;
    const auto t_read = std::chrono::steady_clock::now();
    HostVolume hv = read_volume(filename, parameters, minimum, maximum);
    if (timing)
        std::cout << "RUNTIME of reading the dataset: "
                  << std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_read).count()
                  << " ms" << std::endl;
    Stream stream;
    void *S = (void *)stream.s;
    StageTimer tm(timing, stream.s);
    tm.start();
    DevBuf raw(hv.bytes);
    check_cuda(cudaMemcpyAsync(raw.p, hv.data.get(), hv.bytes, cudaMemcpyHostToDevice, stream.s), "upload");
    std::cout << "Dataset of size " << hv.size.x << " " << hv.size.y << " " << hv.size.z << " loaded" << std::endl;
    tm.stop("of data transfer to device");
    tm.start();
    int box[6];
    const SIPL::int3 shift = input_box(parameters, hv, raw.p, stream.s, box);
    const int X = box[3], Y = box[4], Z = box[5];
    const size_t n = (size_t)X * Y * Z;
    if (X != hv.size.x || Y != hv.size.y || Z != hv.size.z) {
        DevBuf cropped(n * hv.elem);
        check(tsf_crop_copy(raw.p, hv.type, hv.size.x, hv.size.y, hv.size.z, box, cropped.p, S), "cropping");
        raw.swap(cropped);
    }
    tm.stop("of cropping");
    hv.data.reset();   // the upload has been staged; the host copy is not needed again
    const bool tdf16 = getParamBool(parameters, "16bit-vectors");
    const int st = storage_from_parameters(parameters);

    TSFOutput *output = new TSFOutput(new SIPL::int3(X, Y, Z), tdf16);
    output->setSpacing(hv.spacing);
    output->setShiftVector(shift);
    try {
        tm.start();
        DevBuf vol(n * 4);
        check(tsf_to_float(raw.p, hv.type, (int64_t)n, minimum, maximum, vol.as<float>(), S), "toFloat");
        raw.alloc(0);
        tm.stop("of to float conversion");

        FieldResult fr;
        circle_fitting_method(parameters, vol.as<float>(), X, Y, Z, st, tdf16, stream.s, tm, fr);
        vol.alloc(0);
        check_cuda(cudaStreamSynchronize(stream.s), "TDF");
        void *d_T = fr.T.p;                      // the output owns it from here on
        output->setDeviceTDF(fr.T.release());
        if (getParamBool(parameters, "tdf-only")) return output;

        // runNewCenterlineAlg, front half (parallelCenterlineExtraction.cpp:667-899)
        tm.start();
        const size_t wsb = tsf_candidates_workspace_size(X, Y, Z);
        const int64_t max_vertices = 16384;
        DevBuf ws(wsb), cp(n), verts(sizeof(int32_t) * 3 * max_vertices);
        int64_t nc = 0, nv = 0;
        const int code = tsf_candidates(d_T, tdf16, fr.R.as<float>(), fr.field.p, st, X, Y, Z,
                                        getParam(parameters, "tdf-high"), (int)getParam(parameters, "cube-size"),
                                        verts.as<int32_t>(), max_vertices, cp.as<int8_t>(), nullptr, 0, &nc, &nv,
                                        ws.p, wsb, S);
        std::cout << "candidates: " << nc << std::endl;
        if (nc <= 0 || (double)nc > 0.5 * (double)n)
            throw SIPL::SIPLException("The number of candidate voxels is too low or too high. Something went "
                                      "wrong... Wrong parameters? Out of memory?", __LINE__, __FILE__);
        if (getParamBool(parameters, "centerpoints-only")) {
            check_cuda(cudaStreamSynchronize(stream.s), "candidates");
            output->setDeviceCenterlineVoxels(static_cast<int8_t *>(cp.release()));
            return output;
        }
        std::cout << "number of vertices detected " << nv << std::endl;
        if (code != TSF_OK && code != TSF_ERR_COUNT_RANGE) check(code, "candidates");
        if (nv < 8) throw SIPL::SIPLException("Too few centerpoints detected. Revise parameters.", __LINE__, __FILE__);
        if (nv >= 16384)
            throw SIPL::SIPLException("Too many centerpoints detected. More cropping of dataset is probably needed.",
                                      __LINE__, __FILE__);
        std::vector<int32_t> hv3((size_t)nv * 3);
        check_cuda(cudaMemcpyAsync(hv3.data(), verts.p, hv3.size() * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                   stream.s), "vertices");
        check_cuda(cudaStreamSynchronize(stream.s), "vertices");
        std::vector<SIPL::int3> vlist((size_t)nv);
        for (int64_t i = 0; i < nv; i++) vlist[(size_t)i] = SIPL::int3(hv3[3 * i], hv3[3 * i + 1], hv3[3 * i + 2]);
        output->setCenterpoints(vlist);
        tm.stop("centerpoint extraction");

        // runNewCenterlineAlg, back half (parallelCenterlineExtraction.cpp:911-1332)
        tm.start();
        const int nvi = (int)nv;
        const size_t lwb = tsf_link_workspace_size(nvi);
        DevBuf lws(lwb), dedges(sizeof(int32_t) * 4 * (size_t)nvi), dlabels(sizeof(int32_t) * (size_t)nvi),
            dsizes(sizeof(int32_t) * (size_t)nvi);
        int ne = 0;
        const int lcode = tsf_link_centerpoints(verts.as<int32_t>(), nvi, d_T, tdf16, X, Y, Z,
                                                getParam(parameters, "min-mean-tdf"),
                                                getParam(parameters, "max-distance"), dedges.as<int32_t>(), &ne,
                                                dlabels.as<int32_t>(), dsizes.as<int32_t>(), lws.p, lwb, S);
        std::cout << "number of edges detected " << ne << std::endl;
        if (lcode == TSF_ERR_COUNT_RANGE) throw SIPL::SIPLException("No edges were found", __LINE__, __FILE__);
        check(lcode, "linking");
        tm.stop("linking");
        tm.start();
        const int min_tree = (int)getParam(parameters, "min-tree-length");
        const std::string vtk = getParamStr(parameters, "centerline-vtk-file");
        const bool segment = !getParamBool(parameters, "no-segmentation");
        const int8_t *d_cl = nullptr;   // the centerlines on the device, for the segmentation
        if (vtk != "off" || getParamBool(parameters, "loop-removal")) {
            // host loop removal (parallelCenterlineExtraction.cpp:1168-1247); the centerline voxels and
            // the radius smoothing of createCenterlineVoxels (:287-321) touch only the cells along the kept
            // edges, which are read from and written to the device volumes (the reference writes the
            // centerlines and the averaged radius back to its images, :1235-1249)
            std::vector<int32_t> he(2 * (size_t)ne), hl((size_t)nvi), hs((size_t)nvi);
            check_cuda(cudaMemcpyAsync(he.data(), dedges.p, he.size() * 4, cudaMemcpyDeviceToHost, stream.s), "edges");
            check_cuda(cudaMemcpyAsync(hl.data(), dlabels.p, hl.size() * 4, cudaMemcpyDeviceToHost, stream.s), "labels");
            check_cuda(cudaMemcpyAsync(hs.data(), dsizes.p, hs.size() * 4, cudaMemcpyDeviceToHost, stream.s), "sizes");
            check_cuda(cudaStreamSynchronize(stream.s), "graph download");
            const int split = vtk != "off" ? (int)getParam(parameters, "max-edge-distance") : 0;
            StageTimer graph_tm(tm.on(), stream.s);
            graph_tm.host_start();
            int cap = 4 * (nvi + ne) + 1024, nov = 0, noe = 0, gcode;
            int64_t ccap = 16 * (int64_t)cap, nc = 0;
            std::vector<int32_t> ov, oe;
            std::vector<int64_t> cells, start;
            for (;;) {
                ov.assign(3 * (size_t)cap, 0);
                oe.assign(2 * (size_t)cap, 0);
                cells.resize((size_t)ccap);
                start.resize((size_t)cap + 1);
                gcode = tsf_centerline_graph_cells(hv3.data(), nvi, he.data(), ne, hl.data(), hs.data(), min_tree,
                                                   split, X, Y, Z, ov.data(), oe.data(), cap, &nov, &noe,
                                                   cells.data(), start.data(), ccap, &nc);
                if (gcode != TSF_ERR_CAPACITY) break;
                cap = std::max(cap, 2 * std::max(nov, noe));
                ccap = std::max(ccap, 2 * nc);
            }
            if (gcode == TSF_ERR_COUNT_RANGE)
                throw SIPL::SIPLException("Centerline graph size is 0! Can't continue. Maybe lower min-tree-length?",
                                          __LINE__, __FILE__);
            check(gcode, "centerline graph");
            DevBuf dcells(sizeof(int64_t) * (size_t)std::max<int64_t>(nc, 1)),
                dvals(sizeof(float) * (size_t)std::max<int64_t>(nc, 1));
            std::vector<float> vals((size_t)nc);
            check_cuda(cudaMemcpyAsync(dcells.p, cells.data(), sizeof(int64_t) * (size_t)nc, cudaMemcpyHostToDevice,
                                       stream.s), "cells");
            check(tsf_gather_cells(fr.R.as<float>(), X, Y, Z, dcells.as<int64_t>(), nc, dvals.as<float>(), S),
                  "radius");
            check_cuda(cudaMemcpyAsync(vals.data(), dvals.p, sizeof(float) * (size_t)nc, cudaMemcpyDeviceToHost,
                                       stream.s), "radius");
            check_cuda(cudaStreamSynchronize(stream.s), "radius");
            std::vector<int64_t> ucells((size_t)nc);
            std::vector<float> uvals((size_t)nc);
            int64_t nu = 0;
            check(tsf_centerline_smooth_radius(cells.data(), start.data(), noe, vals.data(), ucells.data(),
                                               uvals.data(), &nu), "centerline radius");
            graph_tm.host_stop("of loop removal and centerline voxels (host)");
            DevBuf cl(n);
            check_cuda(cudaMemsetAsync(cl.p, 0, n, stream.s), "centerlines");
            check_cuda(cudaMemcpyAsync(dcells.p, ucells.data(), sizeof(int64_t) * (size_t)nu, cudaMemcpyHostToDevice,
                                       stream.s), "cells");
            check_cuda(cudaMemcpyAsync(dvals.p, uvals.data(), sizeof(float) * (size_t)nu, cudaMemcpyHostToDevice,
                                       stream.s), "radius");
            check(tsf_centerline_apply(cl.as<int8_t>(), segment ? fr.R.as<float>() : nullptr, X, Y, Z,
                                       dcells.as<int64_t>(), dvals.as<float>(), nu, S), "centerlines");
            check_cuda(cudaStreamSynchronize(stream.s), "centerlines");
            d_cl = cl.as<int8_t>();        // owned by the output from here on
            output->setDeviceCenterlineVoxels(static_cast<int8_t *>(cl.release()));
            if (vtk != "off" && tsf_write_centerline_vtk(vtk.c_str(), ov.data(), nov, oe.data(), noe) != TSF_OK)
                throw SIPL::IOException(vtk.c_str(), __LINE__, __FILE__);
        } else {
            // removeSmallTrees on the GPU (kernels.cl:510-534)
            DevBuf cl(n);
            check_cuda(cudaMemsetAsync(cl.p, 0, n, stream.s), "centerlines");
            check(tsf_rasterize_trees(verts.as<int32_t>(), dedges.as<int32_t>(), ne, dlabels.as<int32_t>(),
                                      dsizes.as<int32_t>(), min_tree, cl.as<int8_t>(), X, Y, Z, S),
                  "rasterise trees");
            check_cuda(cudaStreamSynchronize(stream.s), "centerlines");
            d_cl = cl.as<int8_t>();        // owned by the output from here on
            output->setDeviceCenterlineVoxels(static_cast<int8_t *>(cl.release()));
        }
        tm.stop("of removing small trees");
        // runInverseGradientSegmentation / runSphereSegmentation (tube-segmentation.cpp:967-976)
        if (segment) {
            tm.start();
            DevBuf seg(n);
            if (!getParamBool(parameters, "sphere-segmentation")) {
                const size_t swb = tsf_segment_workspace_size(X, Y, Z);
                DevBuf sws(swb);
                int iters = 0;
                check(tsf_segment_inverse_gradient(d_cl, fr.field.p, st, fr.R.as<float>(), X, Y, Z,
                                                   seg.as<int8_t>(), &iters, sws.p, swb, S),
                      "segmentation");
                std::cout << "segmentation result grown in " << iters << " iterations" << std::endl;
            } else {
                check(tsf_segment_spheres(d_cl, fr.R.as<float>(), X, Y, Z, seg.as<int8_t>(), S), "segmentation");
            }
            check_cuda(cudaStreamSynchronize(stream.s), "segmentation");
            output->setDeviceSegmentation(static_cast<int8_t *>(seg.release()));
            tm.stop("of segmentation");
        }
        if (getParamStr(parameters, "storage-dir") != "off")
            writeDataToDisk(output, getParamStr(parameters, "storage-dir"), getParamStr(parameters, "storage-name"));
        return output;
    } catch (...) {
        delete output;
        throw;
    }
}

TSFOutput *runSegmentation(std::string filename, paramList &parameters, std::string kernel_dir) {
    return run(filename, parameters, kernel_dir);
}
