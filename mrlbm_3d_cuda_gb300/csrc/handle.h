// Host-side state behind the C ABI: the handle (one case on the device) and the batch.
// Shared by the host translation units of the library (api.cpp, output.cpp).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "kernels.h"
#include "lattice_tables.h"
#include "mrlbm_internal.h"

namespace mrlbm {
extern thread_local std::string g_last_error;
constexpr int kRing = 65536;  // sampled steps kept on the device (forces, diagnostics)
constexpr int kWatchdogDefault = 64;  // steps between divergence checks unless the case sets it
}  // namespace mrlbm

using mrlbm::BatchArgs;
using mrlbm::Derived;
using mrlbm::Geometry;
using mrlbm::StepArgs;
using mrlbm::StorageScale;

struct mrlbm_handle {
    mrlbm_case_desc d{};
    Derived der{};
    Geometry geo;
    std::string err;
    bool host_only = false;
    int dev = 0, n_sm = 0;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    // the boundary-tile step launch runs beside the bulk one: side stream and fork / join events
    cudaStream_t side_stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int storage = 0, vbytes = 4;
    StorageScale sc{};
    int64_t n = 0, fs = 0;
    void *m[2] = {nullptr, nullptr};
    int parity = 0;
    bool initialized = false;
    int64_t step = 0;
    // step-kernel configuration
    int tile_y = 8, lz = 32, tiles_x = 0, tiles_y = 0, n_items = 0, n_ctas = 0;
    int64_t n_fluid = 0;
    uint32_t *d_word = nullptr;
    int32_t *d_items = nullptr, *d_tile_slot = nullptr;
    float *d_side = nullptr;
    int n_special = 0;
    // non-bulk node list handled by the node-list kernel
    uint64_t *d_list_xyz = nullptr;
    uint32_t *d_list_word = nullptr;
    int32_t *d_row_base = nullptr;
    float *d_popbuf = nullptr;
    int n_list_pop = 0, n_list = 0, n_list_blocks = 0;
    // walls
    float *d_wf[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
    uint32_t *d_wm[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    int64_t *d_wl[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    uint32_t *d_tag = nullptr;  // [512]: in masks then out masks
    StepArgs args{};
    StepArgs *d_args = nullptr;     // work items of tiles without boundary nodes (bulk kernel)
    StepArgs *d_args_sp = nullptr;  // the same with the work items of tiles holding boundary nodes
    int n_items_sp = 0, n_ctas_sp = 0;
    std::vector<int32_t> h_items, h_items_sp;  // host copies of the two work-item lists
    mrlbm_batch *batch = nullptr;   // owning batch, if any
    int *d_error = nullptr;
    // divergence watchdog: every watchdog_every steps (0: off) the step computes its FP64 mass /
    // energy sums into d_watch and flags non-finite ones in the error word, whose value is then
    // copied to the pinned word h_status; mrlbm_step reads h_status without a synchronisation
    int watchdog_every = 0;
    double *d_watch = nullptr;
    int *h_status = nullptr;
    uint32_t *d_sr_step = nullptr;  // stochastic-rounding step counter (16-bit storage with it on)
    // sampling
    int force_every = 0, diag_every = 0;
    double *d_force_ring = nullptr, *d_diag_ring = nullptr, *d_diag_part = nullptr;
    std::vector<int64_t> force_steps, diag_steps;
    int64_t forces_written = 0;  // force samples already written by mrlbm_write_forces
    // time-averaged wall pressure (pressure.dat)
    int64_t ps_start = -1, ps_end = -1;
    int ps_count = 0;
    double *d_ps_avg[2] = {nullptr, nullptr};
    // inlet density of the statistics window: [0] running mean, then per sample (rho_in, mean
    // over the earlier samples); inlet_steps holds the step of each ring slot
    double *d_inlet = nullptr;
    std::vector<int64_t> inlet_steps;
    int64_t inlet_written = 0;
    int64_t force_count = 0, diag_count = 0;
    // staging
    float *d_stage = nullptr;
    size_t stage_bytes = 0;
};

// Independent cases advanced together: every step is one persistent step-kernel launch over
// the work items of all cases, one node-list launch and one wall launch, replayed from CUDA
// graphs (one per ping-pong parity and force sampling).
struct mrlbm_batch {
    std::vector<mrlbm_handle *> h;
    cudaStream_t stream = nullptr;
    cudaStream_t side_stream = nullptr;  // boundary-tile step launch, forked / joined by events
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int storage = 0, tile_y = 16, lz = 0;
    int parity = 0;
    int64_t step = 0;
    int force_every = 0;
    int64_t force_count = 0;  // sampled steps so far (the ring slot of the cases with walls)
    // device tables (BatchArgs and what it points to)
    const StepArgs **d_cases = nullptr;
    int2 *d_items = nullptr;  // bulk work items, then the boundary-tile work items
    int4 *d_list_blocks = nullptr, *d_wall_blocks = nullptr;
    double **d_ring = nullptr;
    int *d_slot = nullptr;
    BatchArgs *d_ba = nullptr, *d_ba_sp = nullptr;  // bulk / boundary-tile items
    int n_items = 0, n_ctas = 0, n_items_sp = 0, n_ctas_sp = 0, n_list_blocks = 0, n_wall_blocks = 0;
    int *d_work = nullptr;  // [2] work-item counters of the two batched step launches
    cudaGraphExec_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [parity][force]
};



namespace mrlbm {
// Record an error on the handle (if any) and as this thread's last error; returns `code`.
int fail(mrlbm_handle *h, int code, const std::string &msg);
int cuda_fail(mrlbm_handle *h, cudaError_t e, const char *what);
// Device staging buffer of at least `bytes` (FP32 host-layout conversions).
int ensure_stage(mrlbm_handle *h, size_t bytes);
// Set the stochastic-rounding step counter to the handle's step (after init, load, restore).
int sync_sr_step(mrlbm_handle *h);
// Clear the divergence flag of the device error word and its host copy (new state).
int clear_divergence(mrlbm_handle *h);
}  // namespace mrlbm

#define CK(h, call)                                                    \
    do {                                                               \
        cudaError_t e_ = (call);                                       \
        if (e_ != cudaSuccess) return mrlbm::cuda_fail(h, e_, #call);  \
    } while (0)
