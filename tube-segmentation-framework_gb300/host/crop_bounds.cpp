// crop_bounds.cpp -- the host half of the cropping stage: the crop box from
// the per-slice scan-line counts, and the fixed in-plane crop of the
// AAA-Vessels-CT preset (readDatasetAndTransfer, tube-segmentation.cpp:1611-1772).
#include <cmath>
#include <string>

#include "tsf/tsf_c.h"

namespace tsf {
int fail(int code, const std::string &msg);
}

// Round an extent to a multiple of 4 inside the volume: widen alternately
// below and above (the alternation carries over from one axis to the next, as
// in the reference), then shrink from above if the volume is too small.
static void round_to_4(int &lo, int &hi, int &size, int full, bool &lower) {
    while (size % 4 != 0 && size < full) {
        if (lower && lo > 0) lo--;
        else if (hi < full) hi++;
        lower = !lower;
        size = hi - lo;
    }
    while (size % 4 != 0) size--;
}

extern "C" int tsf_crop_bounds(const int16_t *counts, int X, int Y, int Z, int min_scan_lines, int start_z_middle,
                               int *box) {
    if (!counts || !box) return tsf::fail(TSF_ERR_INVALID_ARG, "null buffer");
    if (X <= 0 || Y <= 0 || Z <= 0) return tsf::fail(TSF_ERR_INVALID_ARG, "bad volume extents");
    const int16_t *cx = counts, *cy = counts + X, *cz = counts + X + Y;
    int x1 = 0, x2 = X, y1 = 0, y2 = Y, z1 = 0, z2 = Z;
    // first and last slice with more than min_scan_lines inside (the last
    // search stops before slice 0 and keeps the full extent when nothing is found)
    for (int s = 0; s < X; s++)
        if (cx[s] > min_scan_lines) { x1 = s; break; }
    for (int s = X - 1; s > 0; s--)
        if (cx[s] > min_scan_lines) { x2 = s; break; }
    for (int s = 0; s < Y; s++)
        if (cy[s] > min_scan_lines) { y1 = s; break; }
    for (int s = Y - 1; s > 0; s--)
        if (cy[s] > min_scan_lines) { y2 = s; break; }
    // z: from the middle outwards to the first slice with fewer lines inside
    // ("middle", the lung cropping), or like x and y ("end")
    const int start = start_z_middle ? Z / 2 : 0, a = start_z_middle ? -1 : 1;
    for (int s = start; s < Z; s++)
        if (a * cz[s] > a * min_scan_lines) { z2 = s; break; }
    for (int s = Z - start - 1; s > 0; s--)
        if (a * cz[s] > a * min_scan_lines) { z1 = s; break; }
    if (!start_z_middle) {
        const int t = z1;
        z1 = z2;
        z2 = t;
    }
    int SX = x2 - x1, SY = y2 - y1, SZ = z2 - z1;
    if (SX <= 0 || SY <= 0 || SZ <= 0)
        return tsf::fail(TSF_ERR_INVALID_ARG, "Invalid cropping to new size " + std::to_string(SX) + ", " +
                                                  std::to_string(SY) + ", " + std::to_string(SZ));
    bool lower = false;
    round_to_4(x1, x2, SX, X, lower);
    round_to_4(y1, y2, SY, Y, lower);
    round_to_4(z1, z2, SZ, Z, lower);
    if (SX <= 0 || SY <= 0 || SZ <= 0)
        return tsf::fail(TSF_ERR_INVALID_ARG, "Invalid cropping to new size " + std::to_string(SX) + ", " +
                                                  std::to_string(SY) + ", " + std::to_string(SZ));
    box[0] = x1;
    box[1] = y1;
    box[2] = z1;
    box[3] = SX;
    box[4] = SY;
    box[5] = SZ;
    return TSF_OK;
}

extern "C" int tsf_crop_box_fixed(int X, int Y, int Z, float fraction, int *box) {
    if (!box) return tsf::fail(TSF_ERR_INVALID_ARG, "null buffer");
    const int ox = (int)std::round((float)X * fraction), oy = (int)std::round((float)Y * fraction);
    int SX = X - 2 * ox, SY = Y - 2 * oy, SZ = Z;
    if (SX <= 0 || SY <= 0) return tsf::fail(TSF_ERR_INVALID_ARG, "volume too small for the crop");
    SX -= SX % 4;
    SY -= SY % 4;
    SZ -= SZ % 4;
    if (SX <= 0 || SY <= 0 || SZ <= 0) return tsf::fail(TSF_ERR_INVALID_ARG, "volume too small for the crop");
    box[0] = ox;
    box[1] = oy;
    box[2] = 0;
    box[3] = SX;
    box[4] = SY;
    box[5] = SZ;
    return TSF_OK;
}
