// SIPL/Types.hpp -- the small vector types of the reference's API
// (SIPL::int3, SIPL::float3, SIPL::int2).
#ifndef TSF_SIPL_TYPES_HPP
#define TSF_SIPL_TYPES_HPP

#include <cmath>

namespace SIPL {

struct int2 {
    int x = 0, y = 0;
    int2() = default;
    int2(int x_, int y_) : x(x_), y(y_) {}
};

struct int3 {
    int x = 0, y = 0, z = 0;
    int3() = default;
    int3(int x_, int y_, int z_) : x(x_), y(y_), z(z_) {}
    bool operator==(const int3 &o) const { return x == o.x && y == o.y && z == o.z; }
    float distance(const int3 &o) const {
        const float dx = (float)(x - o.x), dy = (float)(y - o.y), dz = (float)(z - o.z);
        return std::sqrt(dx * dx + dy * dy + dz * dz);
    }
};

struct float3 {
    float x = 0, y = 0, z = 0;
    float3() = default;
    float3(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
    float length() const { return std::sqrt(x * x + y * y + z * z); }
};

}  // namespace SIPL
#endif
