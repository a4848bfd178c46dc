// inputOutput.hpp -- TSFOutput, the result container of run() (reference
// inputOutput.hpp:10-52, inputOutput.cpp:66-239), and the result writers.
//
// Same public members as the reference except the OpenCL-typed ones: the
// cl::Image3D setters are replaced by device-buffer setters (CUDA device
// memory owned by the object), getContext() is dropped, and the
// oul::DeviceCriteria constructor argument is accepted for source
// compatibility (a GPU is always used).  Host getters copy device results to
// the host lazily on first use; a unorm16 TDF is converted to float by
// dividing by 65535, as the reference does.  The object owns every array it
// holds and frees it in its destructor, including the size pointer.
#ifndef TSF_INPUT_OUTPUT_HPP
#define TSF_INPUT_OUTPUT_HPP

#include <cstdint>
#include <string>
#include <vector>

#include "tsf/SIPL/Types.hpp"
#include "tsf/parameters.hpp"

namespace oul {
enum DeviceType { DEVICE_TYPE_ANY, DEVICE_TYPE_GPU, DEVICE_TYPE_CPU };
// Accepted for source compatibility with code written against the reference;
// device selection is the current CUDA device.
class DeviceCriteria {
public:
    void setTypeCriteria(DeviceType t) { type = t; }
    void setDeviceCountCriteria(int n) { count = n; }
    DeviceType type = DEVICE_TYPE_ANY;
    int count = 1;
};
}  // namespace oul

class TSFOutput {
public:
    TSFOutput(oul::DeviceCriteria criteria, SIPL::int3 *size, bool TDFis16bit = false);
    explicit TSFOutput(SIPL::int3 *size, bool TDFis16bit = false);
    ~TSFOutput();
    TSFOutput(const TSFOutput &) = delete;
    TSFOutput &operator=(const TSFOutput &) = delete;

    bool hasSegmentation() { return deviceHasSegmentation || hostHasSegmentation; }
    bool hasCenterlineVoxels() { return deviceHasCenterlineVoxels || hostHasCenterlineVoxels; }
    bool hasTDF() { return deviceHasTDF || hostHasTDF; }

    // host data (ownership passes to the object; allocate with new[])
    void setTDF(float *);
    void setSegmentation(char *);
    void setCenterlineVoxels(char *);
    // device data (CUDA device memory allocated with cudaMalloc; ownership
    // passes to the object).  The TDF is float, or uint16 unorm16 when the
    // object was made with TDFis16bit.
    void setDeviceTDF(void *d_tdf);
    void setDeviceSegmentation(int8_t *d_seg);
    void setDeviceCenterlineVoxels(int8_t *d_centerline);

    void setSize(SIPL::int3 *);
    char *getSegmentation();
    char *getCenterlineVoxels();
    float *getTDF();
    SIPL::int3 *getSize();
    SIPL::int3 getShiftVector() const;
    void setShiftVector(SIPL::int3 shiftVector);
    SIPL::float3 getSpacing() const;
    void setSpacing(SIPL::float3 spacing);

    // Centerpoint vertices of the candidate stage, in the reference's
    // histogram-pyramid order (parallelCenterlineExtraction.cpp:884-893).
    const std::vector<SIPL::int3> &getCenterpoints() const { return centerpoints; }
    void setCenterpoints(const std::vector<SIPL::int3> &v) { centerpoints = v; }

private:
    SIPL::int3 *size;
    SIPL::float3 spacing;
    SIPL::int3 shiftVector;
    bool TDFis16bit;
    bool hostHasSegmentation = false, hostHasCenterlineVoxels = false, hostHasTDF = false;
    bool deviceHasTDF = false, deviceHasCenterlineVoxels = false, deviceHasSegmentation = false;
    char *segmentation = nullptr;
    char *centerlineVoxels = nullptr;
    float *TDF = nullptr;
    void *d_TDF = nullptr;
    int8_t *d_segmentation = nullptr;
    int8_t *d_centerline = nullptr;
    std::vector<SIPL::int3> centerpoints;
};

// inputOutput.cpp:14-46: <dir><name>.centerline.mhd/.raw and
// <dir><name>.segmentation.mhd/.raw (MET_CHAR)
void writeDataToDisk(TSFOutput *output, std::string storageDirectory, std::string name);

// inputOutput.cpp:48-64: POLYDATA with the vertices and edges
void writeToVtkFile(paramList &parameters, std::vector<SIPL::int3> vertices, std::vector<SIPL::int2> edges);

#endif
