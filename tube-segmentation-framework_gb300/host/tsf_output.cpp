// tsf_output.cpp -- TSFOutput and the result writers (interface of reference
// inputOutput.hpp / inputOutput.cpp).
#include <cuda_runtime_api.h>

#include <algorithm>
#include <cstdio>
#include <fstream>
#include <memory>
#include <vector>

#include "first_touch.hpp"
#include "tsf/SIPL/Exceptions.hpp"
#include "tsf/inputOutput.hpp"

namespace {

int64_t voxels(const SIPL::int3 *s) { return s ? (int64_t)s->x * s->y * s->z : 0; }

void copy_to_host(void *dst, const void *src, size_t bytes) {
    const cudaError_t e = cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        const std::string msg = std::string("device to host copy failed: ") + cudaGetErrorString(e);
        throw SIPL::SIPLException(msg.c_str(), __LINE__, __FILE__);
    }
}

}  // namespace

TSFOutput::TSFOutput(oul::DeviceCriteria, SIPL::int3 *size_, bool TDFis16bit_)
    : size(size_), spacing(1, 1, 1), TDFis16bit(TDFis16bit_) {}

TSFOutput::TSFOutput(SIPL::int3 *size_, bool TDFis16bit_) : size(size_), spacing(1, 1, 1), TDFis16bit(TDFis16bit_) {}

TSFOutput::~TSFOutput() {
    if (hostHasTDF) delete[] TDF;
    if (hostHasSegmentation) delete[] segmentation;
    if (hostHasCenterlineVoxels) delete[] centerlineVoxels;
    if (d_TDF) cudaFree(d_TDF);
    if (d_segmentation) cudaFree(d_segmentation);
    if (d_centerline) cudaFree(d_centerline);
    delete size;
}

void TSFOutput::setTDF(float *data) {
    if (hostHasTDF && TDF != data) delete[] TDF;
    TDF = data;
    hostHasTDF = true;
}
void TSFOutput::setSegmentation(char *data) {
    if (hostHasSegmentation && segmentation != data) delete[] segmentation;
    segmentation = data;
    hostHasSegmentation = true;
}
void TSFOutput::setCenterlineVoxels(char *data) {
    if (hostHasCenterlineVoxels && centerlineVoxels != data) delete[] centerlineVoxels;
    centerlineVoxels = data;
    hostHasCenterlineVoxels = true;
}
void TSFOutput::setDeviceTDF(void *d) {
    if (d_TDF && d_TDF != d) cudaFree(d_TDF);
    d_TDF = d;
    deviceHasTDF = d != nullptr;
}
void TSFOutput::setDeviceSegmentation(int8_t *d) {
    if (d_segmentation && d_segmentation != d) cudaFree(d_segmentation);
    d_segmentation = d;
    deviceHasSegmentation = d != nullptr;
}
void TSFOutput::setDeviceCenterlineVoxels(int8_t *d) {
    if (d_centerline && d_centerline != d) cudaFree(d_centerline);
    d_centerline = d;
    deviceHasCenterlineVoxels = d != nullptr;
}
void TSFOutput::setSize(SIPL::int3 *s) { size = s; }

float *TSFOutput::getTDF() {
    if (hostHasTDF) return TDF;
    if (!deviceHasTDF) throw SIPL::SIPLException("Trying to fetch non existing data from TSFOutput", __LINE__, __FILE__);
    const int64_t n = voxels(size);
    TDF = new float[n];
    if (TDFis16bit) {
        // the unorm16 TDF read as v / 65535, as the reference's getter does
        // (inputOutput.cpp:164), on up to 16 host threads
        std::unique_ptr<uint16_t[]> tmp(new uint16_t[(size_t)n]);
        tsf_host::parallel_fill(tmp.get(), 0, sizeof(uint16_t) * (size_t)n);
        copy_to_host(tmp.get(), d_TDF, sizeof(uint16_t) * (size_t)n);
        const uint16_t *src = tmp.get();
        float *dst = TDF;
        const int64_t nt = (int64_t)tsf_host::host_threads(sizeof(float) * (size_t)n);
        tsf_host::parallel_tasks((size_t)nt, [=](size_t t) {
            const int64_t i0 = n * (int64_t)t / nt, i1 = n * ((int64_t)t + 1) / nt;
            for (int64_t i = i0; i < i1; i++) dst[i] = (float)src[i] / 65535.0f;
        });
    } else {
        tsf_host::parallel_fill(TDF, 0, sizeof(float) * (size_t)n);
        copy_to_host(TDF, d_TDF, sizeof(float) * (size_t)n);
    }
    hostHasTDF = true;
    return TDF;
}

char *TSFOutput::getSegmentation() {
    if (hostHasSegmentation) return segmentation;
    if (!deviceHasSegmentation)
        throw SIPL::SIPLException("Trying to fetch non existing data from TSFOutput", __LINE__, __FILE__);
    segmentation = new char[voxels(size)];
    tsf_host::parallel_fill(segmentation, 0, (size_t)voxels(size));
    copy_to_host(segmentation, d_segmentation, (size_t)voxels(size));
    hostHasSegmentation = true;
    return segmentation;
}

char *TSFOutput::getCenterlineVoxels() {
    if (hostHasCenterlineVoxels) return centerlineVoxels;
    if (!deviceHasCenterlineVoxels)
        throw SIPL::SIPLException("Trying to fetch non existing data from TSFOutput", __LINE__, __FILE__);
    centerlineVoxels = new char[voxels(size)];
    tsf_host::parallel_fill(centerlineVoxels, 0, (size_t)voxels(size));
    copy_to_host(centerlineVoxels, d_centerline, (size_t)voxels(size));
    hostHasCenterlineVoxels = true;
    return centerlineVoxels;
}

SIPL::int3 *TSFOutput::getSize() { return size; }
SIPL::int3 TSFOutput::getShiftVector() const { return shiftVector; }
void TSFOutput::setShiftVector(SIPL::int3 v) { shiftVector = v; }
SIPL::float3 TSFOutput::getSpacing() const { return spacing; }
void TSFOutput::setSpacing(SIPL::float3 s) { spacing = s; }

static void write_mhd_raw(TSFOutput *out, const std::string &dir, const std::string &name, const char *what,
                          const char *data) {
    const SIPL::int3 *s = out->getSize();
    const SIPL::float3 sp = out->getSpacing();
    const std::string base = name + "." + what;
    std::ofstream mhd((dir + base + ".mhd").c_str());
    if (!mhd.is_open()) throw SIPL::IOException((dir + base + ".mhd").c_str());
    mhd << "ObjectType = Image\nNDims = 3\n";
    mhd << "DimSize = " << s->x << " " << s->y << " " << s->z << "\n";
    mhd << "ElementSpacing = " << sp.x << " " << sp.y << " " << sp.z << "\n";
    mhd << "ElementType = MET_CHAR\nElementDataFile = " << base << ".raw\n";
    FILE *f = std::fopen((dir + base + ".raw").c_str(), "wb");
    if (!f) throw SIPL::IOException((dir + base + ".raw").c_str());
    std::fwrite(data, 1, (size_t)s->x * s->y * s->z, f);
    std::fclose(f);
}

void writeDataToDisk(TSFOutput *output, std::string storageDirectory, std::string name) {
    if (output->hasCenterlineVoxels())
        write_mhd_raw(output, storageDirectory, name, "centerline", output->getCenterlineVoxels());
    if (output->hasSegmentation())
        write_mhd_raw(output, storageDirectory, name, "segmentation", output->getSegmentation());
}

void writeToVtkFile(paramList &parameters, std::vector<SIPL::int3> vertices, std::vector<SIPL::int2> edges) {
    std::ofstream file(getParamStr(parameters, "centerline-vtk-file").c_str());
    file << "# vtk DataFile Version 3.0\nvtk output\nASCII\n";
    file << "DATASET POLYDATA\nPOINTS " << vertices.size() << " int\n";
    for (const auto &v : vertices) file << v.x << " " << v.y << " " << v.z << "\n";
    file << "\nLINES " << edges.size() << " " << edges.size() * 3 << "\n";
    for (const auto &e : edges) file << "2 " << e.x << " " << e.y << "\n";
}
