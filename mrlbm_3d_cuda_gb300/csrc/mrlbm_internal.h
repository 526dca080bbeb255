// Internal declarations shared by the host (C++) and device (CUDA) parts of libmrlbm.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/mrlbm.h"
#include "lattice_tables.h"

namespace mrlbm {

// Node classes: the numeric values of the reference's NodeTypeEnum
// (MRLBM_3D/src/common/nodeTypeMap.cuh:23-72).  They are part of the exported node-type
// encoding (class << 20 | payload), so they must keep these values.
enum NodeClass : uint32_t {
    C_BULK = 0, C_SOLID, C_INNER, C_OUTER, C_BCFLUID_INNER, C_BCFLUID_OUTER,
    C_BCSOLID_INNER, C_BCSOLID_OUTER,
    C_NORTH, C_SOUTH, C_EAST, C_WEST, C_FRONT, C_BACK,
    C_NORTH_EAST, C_NORTH_WEST, C_NORTH_FRONT, C_NORTH_BACK,
    C_SOUTH_EAST, C_SOUTH_WEST, C_SOUTH_FRONT, C_SOUTH_BACK,
    C_EAST_FRONT, C_EAST_BACK, C_WEST_FRONT, C_WEST_BACK,
    C_NORTH_WEST_FRONT, C_NORTH_WEST_BACK, C_SOUTH_WEST_FRONT, C_SOUTH_WEST_BACK,
    C_NORTH_EAST_FRONT, C_NORTH_EAST_BACK, C_SOUTH_EAST_FRONT, C_SOUTH_EAST_BACK,
    C_COUNT
};

// Internal node word (device): bits 0-5 class, bit 6 frozen (node of a reference block that
// the reference never updates), bit 7 stencil (its post-stream moments feed a curved-wall
// interpolation), bits 8-31 payload (boundary index for INNER/OUTER, octant tag for BCFLUID).
constexpr uint32_t NW_CLASS_MASK = 0x3Fu;
constexpr uint32_t NW_FROZEN = 1u << 6;
constexpr uint32_t NW_STENCIL = 1u << 7;
constexpr int NW_PAYLOAD_SHIFT = 8;

inline uint32_t make_word(uint32_t cls, uint32_t payload, bool frozen, bool stencil) {
    return cls | (frozen ? NW_FROZEN : 0u) | (stencil ? NW_STENCIL : 0u) | (payload << NW_PAYLOAD_SHIFT);
}

// Step-kernel tiling: a CTA owns a TILE_X x tile_y column of nodes and marches along z.
constexpr int TILE_X = 32;

struct WallData {
    std::vector<int64_t> list;       // lexicographic node index, reference scan order
    std::vector<float> nx, ny, delta;
    std::vector<uint32_t> in_mask, out_mask;
    std::vector<int64_t> fluid_list; // BCFLUID nodes of this wall, scan order
    std::vector<int64_t> solid_list; // BCSOLID nodes of this wall (z walls only), scan order
};

// Result of the host classification (lexicographic node order idx = x + nx*(y + ny*z)).
struct Geometry {
    int nx = 0, ny = 0, nz = 0;
    std::vector<uint8_t> cls;       // NodeClass per node
    std::vector<uint32_t> payload;  // boundary index or BCFLUID / BCSOLID tag
    std::vector<uint8_t> frozen;    // node of an all-solid reference block column
    std::vector<uint8_t> stencil;   // needs its post-stream moments kept for the wall kernel
    WallData wall[2];
    uint32_t tag_in_mask[256] = {0};
    uint32_t tag_out_mask[256] = {0};
    int n_walls = 0;
};

// Fill `g` from the descriptor (restating cases/*/nodeClass.cuh and cylinder_helpers.cuh).
// Returns an empty string on success, else an error message.
std::string classify(const mrlbm_case_desc &d, Geometry &g);

// Reference IDX_BLOCK (MRLBM_3D/src/core/index.cuh:11-28) for an nx x ny x nz grid.
MRLBM_HD inline int64_t ref_tiled_index(int x, int y, int z, int nx, int ny) {
    const int64_t gx = (nx + 7) / 8, gy = (ny + 7) / 8;
    const int64_t block = (x / 8) + gx * ((y / 8) + gy * (z / 4));
    const int64_t thread = (x % 8) + 8 * ((y % 8) + 8 * (z % 4));
    return thread + 256 * block;
}

// Host-side derived constants (float / double mix as the reference's constexpr headers).
struct Derived {
    float omega;
    float tau;
};
std::string derive(mrlbm_case_desc &d, Derived &out);

}  // namespace mrlbm
