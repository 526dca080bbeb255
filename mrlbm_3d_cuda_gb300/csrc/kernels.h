// Launch interface between the host runtime (api.cpp) and the CUDA kernels.
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

namespace mrlbm {

// x-blocked, field-interleaved moment layout (see storage.cuh): each 32-node run of an
// (y, z) row owns 10 x 32 consecutive elements.  `esz` is the element size: 4-byte storage
// keeps one field per 32-node line; 2-byte storage keeps the field pairs (2j, 2j+1) of a node
// in one 32-bit word, so a lane moves two fields per access.  aos_index is the element of a
// node's field 0, field_offset the distance of field k from it.
// The hybrid storage mode (FP32 velocity, FP16 density deviation and second moments) keeps
// 7 words per node: ux, uy, uz as FP32, then the FP16 pairs (rho - rho0, mxx), (myy, mzz),
// (mxy, mxz), (myz, unused).  HybridWord is its 32-bit storage element.
constexpr int kXBlock = 32;
struct HybridWord {
    uint32_t bits;
};
template <typename S>
struct StorageLayout {
    static constexpr int esz = (int)sizeof(S);  // bytes per storage element
    static constexpr int per_node = 10;         // elements per node (32-node run: per_node x 32)
};
template <>
struct StorageLayout<HybridWord> {
    static constexpr int esz = 4;
    static constexpr int per_node = 7;
};
inline __host__ __device__ int64_t aos_index(int x, int y, int z, int nxb, int ny, int esz, int per_node = 10) {
    const int64_t run = ((((int64_t)z * ny + y) * nxb + (x >> 5)) * per_node) * kXBlock;
    return run + (esz == 4 ? (x & (kXBlock - 1)) : 2 * (x & (kXBlock - 1)));
}
template <typename S>
inline __host__ __device__ int64_t aos_at(int x, int y, int z, int nxb, int ny) {
    return aos_index(x, y, z, nxb, ny, StorageLayout<S>::esz, StorageLayout<S>::per_node);
}
inline __host__ __device__ constexpr int field_offset(int k, int esz) {
    return esz == 4 ? k * kXBlock : (k >> 1) * (2 * kXBlock) + (k & 1);
}
inline __host__ __device__ int64_t aos_elements(int nx, int ny, int nz, int per_node = 10) {
    return (int64_t)nz * ny * ((nx + kXBlock - 1) / kXBlock) * per_node * kXBlock;
}

// Low-precision storage keeps scaled deviations from the rest state: stored = value * scale,
// one scale for rho - rho0, one for u, one for m.
struct StorageScale {
    float s[3];   // multiply on store
    float is[3];  // multiply on load
};

struct WallArgs {
    const float *nx = nullptr, *ny = nullptr, *delta = nullptr;
    const uint32_t *in_mask = nullptr, *out_mask = nullptr;
    const int64_t *list = nullptr;  // lexicographic node index
    const int64_t *fluid_list = nullptr;  // BCFLUID nodes of this wall
    int nb = 0, nbf = 0;
    float r_wall = 0.f;             // 0.5 D of the wall
    float dir = 1.f;                // +1 inner wall (fluid outside), -1 outer wall
    float u_wall[3] = {0.f, 0.f, 0.f};
};

// One copy lives in device memory per handle; kernels receive a pointer to it plus the
// per-step scalars (ping-pong parity, sampling buffers).
struct StepArgs {
    void *m[2] = {nullptr, nullptr};  // ping-pong moment buffers (aos layout)
    int nxb = 0;                      // 32-node x-blocks per row
    const uint32_t *word = nullptr;     // internal node words (lexicographic); null if all bulk
    const int32_t *items = nullptr;     // work items: tile index | (z-segment << 20)
    int n_items = 0;
    const int32_t *tile_slot = nullptr; // per xy tile: -1 plain, >= 0 side-buffer slot
    float *side = nullptr;              // post-stream moments of stencil nodes, 10 floats each
    int nx = 0, ny = 0, nz = 0;
    int tiles_x = 0, tiles_y = 0, tile_y = 8, lz = 32;
    float omega = 1.f, rho0 = 1.f, u_max = 0.f;
    int convective = 0, current_update = 0, bcf_strong = 0, wall_strong = 0;
    float xc = 0.f, yc = 0.f;
    StorageScale sc;
    WallArgs wall[2];
    const uint32_t *tag_in = nullptr, *tag_out = nullptr;  // [256] BCFLUID masks
    int *error = nullptr;     // sticky device error flag
    // non-bulk node list (special tiles only): every entry gets its 27 pulled populations
    // from the step kernel, in (tile slot, z, tile row, x) order (n_list == n_list_pop;
    // plain stencil nodes and solid nodes are updated by the step kernel itself)
    const uint64_t *list_xyz = nullptr;   // x | y << 21 | z << 42
    const uint32_t *list_word = nullptr;  // node word of each entry
    int n_list_pop = 0, n_list = 0;
    float *popbuf = nullptr;              // [27][n_list_pop]
    const int32_t *row_base = nullptr;    // [slot][z][tile row]: first list entry of the row
    int *work_counter = nullptr;          // work items claimed beyond the first gridDim.x (zeroed per launch)
    // stochastic rounding of 16-bit stores: the step counter that seeds the random bits
    // (null: round to nearest)
    const uint32_t *sr_step = nullptr;
};

// Several independent cases advanced together: one step-kernel launch over the work items of
// every case, one node-list launch and one wall launch whose blocks each serve one case.
// Lives in device memory; the kernels read each case's own StepArgs through `cases`.
struct BatchArgs {
    const StepArgs *const *cases = nullptr;  // device StepArgs of each case
    const int2 *items = nullptr;             // {case, tile | z-segment << 20}
    int n_items = 0;
    const int4 *list_blocks = nullptr;       // per node-list block: {case, first block of the case, blocks, 0}
    const int4 *wall_blocks = nullptr;       // per wall block: {case, first block of the case, blocks, 0}
    double *const *force_ring = nullptr;     // per case: force ring of the case
    const int *force_slot = nullptr;         // ring slot of the sampled step
    int *work_counter = nullptr;             // as StepArgs::work_counter, for the batched launch
};

// Per-step launch parameters.
struct StepLaunch {
    const StepArgs *ga = nullptr;  // device copy of the handle's StepArgs
    int parity = 0;                // read m[parity], write m[parity ^ 1]
    double *force = nullptr;       // [2][5] FP64 accumulators of a sampled step, or null
    double *diag_part = nullptr;   // [grid][2] per-CTA mass / energy partials, or null
    int n_ctas = 0;
    bool full_tiles = false;       // every tile whole (nx % 32 == 0, ny % tile_y == 0)
};

// Stencil-buffer index of node (x, y, z) for a special tile slot.
inline __host__ __device__ int64_t side_index(int slot, int x, int y, int z, int x0, int y0, int nz, int tile_x,
                                              int tile_y) {
    return (((int64_t)slot * nz + z) * tile_y + (y - y0)) * tile_x + (x - x0);
}

// storage: 0 f32, 1 f16, 2 bf16
cudaError_t launch_step(const StepLaunch &l, int storage, int tile_y, bool special, cudaStream_t s);
cudaError_t launch_step_batch(const BatchArgs *ba, int parity, int storage, int tile_y, bool special, int n_ctas,
                              cudaStream_t s);
cudaError_t prepare_step_batch(int storage, int tile_y);  // before capturing batched launches
cudaError_t launch_special_list_batch(const BatchArgs *ba, int parity, int force, int storage, int n_blocks,
                                      cudaStream_t s);
cudaError_t launch_wall_batch(const BatchArgs *ba, int parity, int force, int storage, int n_blocks, cudaStream_t s);
// Zero the slot of every case's force ring and publish the slot for the batched wall kernel.
cudaError_t launch_batch_force_begin(double *const *ring, int n_cases, int slot, int *d_slot, cudaStream_t s);
int step_kernel_smem_bytes(int tile_y);
int step_kernel_max_ctas_per_sm(int storage, int tile_y);
// Curved-wall closure + collision for the wall nodes of both walls, plus the force sums.
cudaError_t launch_wall(const StepLaunch &l, int storage, int n_total, cudaStream_t s);
// Closures, stencil snapshots and collision of the listed non-bulk nodes (after launch_step).
int special_list_blocks(int n_list);
cudaError_t launch_special_list(const StepLaunch &l, int storage, int n_blocks, double *diag_part, cudaStream_t s);
// Sum the per-CTA diagnostics partials into out[2] in a fixed order; a non-finite sum sets
// kErrorDiverged in *error (if given).
constexpr int kErrorDiverged = 16;
cudaError_t launch_diag_finalize(const double *part, int n, double *out, int *error, cudaStream_t s);

struct InitArgs {
    void *m_a = nullptr, *m_b = nullptr;  // both ping-pong buffers
    int nx = 0, ny = 0, nz = 0;
    int kind = 0;
    double p[8] = {0};
    float rho0 = 1.f, u_max = 0.f;
    StorageScale sc;
};
cudaError_t launch_init(const InitArgs &a, int storage, cudaStream_t s);
// Advance the stochastic-rounding step counter(s) after a step.
cudaError_t launch_sr_tick(uint32_t *ctr, cudaStream_t s);
cudaError_t launch_sr_tick_cases(const StepArgs *const *cases, int n, cudaStream_t s);

// Convert between device storage and an FP32 staging buffer (lexicographic or reference
// tiled layout).  dir = 0: storage -> f32, 1: f32 -> storage (written to dst_a and dst_b).
cudaError_t launch_convert(const void *src, void *dst_a, void *dst_b, float *f32, uint32_t field_mask,
                           int layout, int nx, int ny, int nz, int storage, const StorageScale &sc, int dir,
                           cudaStream_t s);

// Reference-format outputs (output_kernels.cu).
// Floats of one halo face array of the reference layout (axis 0: X_WEST / X_EAST, 1: Y, 2: Z).
int64_t halo_face_floats(int nx, int ny, int nz, int axis);
// The six face-population arrays of a restart.bin (X_WEST, X_EAST, Y_SOUTH, Y_NORTH, Z_BACK,
// Z_FRONT) rebuilt from the moments in buffer `parity`.
cudaError_t launch_halo_export(const StepArgs *ga, int parity, int storage, int64_t n, float *const faces[6],
                               cudaStream_t s);
// Accumulate the wall pressure of the state in buffer `buf` into a running mean over n_avg samples.
// Inlet (x = 0 face) mean density into slot `slot` of the statistics ring, running mean in state[0].
cudaError_t launch_inlet_density(const StepArgs *ga, int buf, int storage, double *state, int slot, int n_avg,
                                 cudaStream_t s);
cudaError_t launch_surface_pressure(const StepArgs *ga, int buf, int storage, int wall, int nb, double *avg, int n_avg,
                                    cudaStream_t s);

// Allocation-free periodic step (mrlbm_step_periodic_noalloc).  Everything the step kernel
// needs besides the caller's two moment buffers lives in one fixed array in the library's
// device image, laid out as:
//   [0, 1536)            StepArgs
//   [1536, 1552)         mass / energy sums (2 doubles)
//   [1600, 1604)         error word
//   [1604, 1608)         work-item counter of the step kernel
//   [2048, 18432)        per-CTA diagnostics partials, 2 doubles per CTA
//   [18432, 65536)       work items, one int32 each
constexpr int kNoAllocScratchBytes = 64 * 1024;
constexpr int kNoAllocDiagOffset = 1536;
constexpr int kNoAllocErrorOffset = 1600;
constexpr int kNoAllocWorkOffset = 1604;
constexpr int kNoAllocPartOffset = 2048;
constexpr int kNoAllocMaxCtas = 1024;
constexpr int kNoAllocItemsOffset = kNoAllocPartOffset + kNoAllocMaxCtas * 2 * (int)sizeof(double);
constexpr int kNoAllocMaxItems = (kNoAllocScratchBytes - kNoAllocItemsOffset) / (int)sizeof(int32_t);  // 11776
constexpr int kNoAllocTileY = 16;

struct NoAllocStep {
    const float *m_in = nullptr;  // FP32 moments in the x-blocked storage layout
    float *m_out = nullptr;
    int nx = 0, ny = 0, nz = 0;
    float omega = 0.f, rho0 = 1.f;
    double *diag_host = nullptr;  // optional: {mass, kinetic energy} as mrlbm_get_diagnostics
    cudaStream_t stream = nullptr;
};
// Returns an MRLBM_* status; on failure `err` holds the message.
int noalloc_periodic_step(const NoAllocStep &p, std::string &err);

}  // namespace mrlbm
