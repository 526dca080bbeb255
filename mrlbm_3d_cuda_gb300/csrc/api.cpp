// Host runtime behind the C ABI of include/mrlbm.h: case setup, device memory, the time
// loop, sampling and host-facing I/O.  One handle = one case on the current CUDA device,
// one stream; no call exits the process (the reference's checkCudaErrors does,
// MRLBM_3D/src/utils/cudaHelpers.cuh:10-21).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>

#include "handle.h"

using namespace mrlbm;

namespace mrlbm {
thread_local std::string g_last_error;
}  // namespace mrlbm

namespace mrlbm {

int fail(mrlbm_handle *h, int code, const std::string &msg) {
    if (h) h->err = msg;
    g_last_error = msg;
    return code;
}

int cuda_fail(mrlbm_handle *h, cudaError_t e, const char *what) {
    const int code = (e == cudaErrorMemoryAllocation) ? MRLBM_ERR_NOMEM
                     : (e == cudaErrorNoKernelImageForDevice || e == cudaErrorUnsupportedPtxVersion) ? MRLBM_ERR_UNSUPPORTED
                                                                                                      : MRLBM_ERR_CUDA;
    return fail(h, code, std::string(what) + ": " + cudaGetErrorString(e));
}


template <typename T>
cudaError_t upload(T **dptr, const T *host, size_t count) {
    if (count == 0) {
        *dptr = nullptr;
        return cudaSuccess;
    }
    cudaError_t e = cudaMalloc((void **)dptr, count * sizeof(T));
    if (e != cudaSuccess) return e;
    return cudaMemcpy(*dptr, host, count * sizeof(T), cudaMemcpyHostToDevice);
}

void free_all(mrlbm_handle *h) {
    auto f = [](void *p) {
        if (p) cudaFree(p);
    };
    f(h->m[0]);
    f(h->m[1]);
    f(h->d_word);
    f(h->d_items);
    f(h->d_args_sp);
    f(h->d_tile_slot);
    f(h->d_side);
    f(h->d_list_xyz);
    f(h->d_list_word);
    f(h->d_row_base);
    f(h->d_popbuf);
    for (int w = 0; w < 2; ++w) {
        for (int k = 0; k < 3; ++k) f(h->d_wf[w][k]);
        for (int k = 0; k < 2; ++k) f(h->d_wm[w][k]);
        for (int k = 0; k < 2; ++k) f(h->d_wl[w][k]);
    }
    f(h->d_tag);
    f(h->d_args);
    f(h->d_error);
    f(h->d_watch);
    if (h->h_status) cudaFreeHost(h->h_status);
    h->h_status = nullptr;
    f(h->d_sr_step);
    f(h->d_force_ring);
    f(h->d_diag_ring);
    f(h->d_diag_part);
    f(h->d_stage);
    f(h->d_ps_avg[0]);
    f(h->d_ps_avg[1]);
    f(h->d_inlet);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    if (h->side_stream) cudaStreamDestroy(h->side_stream);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
}

int64_t node_index_for_layout(const mrlbm_handle *h, int64_t lex, int layout) {
    if (layout != MRLBM_LAYOUT_REF_TILED) return lex;
    const int nx = h->d.nx, ny = h->d.ny;
    const int x = (int)(lex % nx), y = (int)((lex / nx) % ny), z = (int)(lex / ((int64_t)nx * ny));
    return ref_tiled_index(x, y, z, nx, ny);
}

int ensure_stage(mrlbm_handle *h, size_t bytes) {
    if (h->stage_bytes >= bytes) return MRLBM_OK;
    if (h->d_stage) cudaFree(h->d_stage);
    h->d_stage = nullptr;
    h->stage_bytes = 0;
    CK(h, cudaMalloc((void **)&h->d_stage, bytes));
    h->stage_bytes = bytes;
    return MRLBM_OK;
}

// A new state (init, uploaded moments, loaded checkpoint) starts with a clear divergence flag.
// The stream is drained first so that no queued watchdog copy lands after the clear.
int clear_divergence(mrlbm_handle *h) {
    CK(h, cudaStreamSynchronize(h->stream));
    int e = 0;
    CK(h, cudaMemcpy(&e, h->d_error, sizeof(int), cudaMemcpyDeviceToHost));
    e &= ~kErrorDiverged;
    CK(h, cudaMemcpy(h->d_error, &e, sizeof(int), cudaMemcpyHostToDevice));
    *h->h_status = e;
    return MRLBM_OK;
}

int sync_sr_step(mrlbm_handle *h) {
    if (!h->d_sr_step) return MRLBM_OK;
    const uint32_t v = (uint32_t)h->step;
    CK(h, cudaStreamSynchronize(h->stream));
    CK(h, cudaMemcpy(h->d_sr_step, &v, sizeof(v), cudaMemcpyHostToDevice));
    return MRLBM_OK;
}

// Tile height and z-segment length from MRLBM_TILE_Y / MRLBM_LZ, else the defaults: 32 x 16
// columns (the widest tile amortises the rim rebuild best: at 256^3 FP32 on GB300, 32 x 16 /
// 32 x 8 / 32 x 4 run at 0.36 / 0.42 / 0.47 ms per step) and lz = 0, the heuristic below.
void default_tiling(int &ty, int &lz) {
    const char *ety = std::getenv("MRLBM_TILE_Y");
    const char *elz = std::getenv("MRLBM_LZ");
    ty = ety ? std::atoi(ety) : 16;
    if (ty != 4 && ty != 8 && ty != 16) ty = 16;
    lz = elz ? std::max(1, std::atoi(elz)) : 0;
}

int setup_tiling(mrlbm_handle *h, int ty, int lz);

// Bytes of one storage element: FP32 and the hybrid mode's words 4, FP16 / BF16 halves 2.
int storage_element_bytes(int storage) {
    return storage == MRLBM_STORAGE_F16 || storage == MRLBM_STORAGE_BF16 ? 2 : 4;
}

// (Re)build everything that depends on the step kernel's tiling: tile slots and side buffer,
// the non-bulk node list, work items, grid size and the device StepArgs.  Node words and
// geometry do not depend on it, so the autotuner can switch tilings cheaply.
int setup_tiling(mrlbm_handle *h, int ty, int lz) {
    const mrlbm_case_desc &d = h->d;
    const Geometry &g = h->geo;
    if (ty != 4 && ty != 8 && ty != 16) return fail(h, MRLBM_ERR_INVALID_ARG, "tile height must be 4, 8 or 16");
    CK(h, cudaStreamSynchronize(h->stream));
    for (void **p : {(void **)&h->d_tile_slot, (void **)&h->d_side, (void **)&h->d_items, (void **)&h->d_list_xyz,
                     (void **)&h->d_list_word, (void **)&h->d_row_base, (void **)&h->d_popbuf,
                     (void **)&h->d_diag_part}) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
    h->tile_y = ty;
    h->tiles_x = (d.nx + TILE_X - 1) / TILE_X;
    h->tiles_y = (d.ny + ty - 1) / ty;
    int per_sm = step_kernel_max_ctas_per_sm(h->storage, ty);
    if (per_sm <= 0) per_sm = 1;
    const int resident = per_sm * h->n_sm;
    const int tiles = h->tiles_x * h->tiles_y;
    if (lz > 0) {
        lz = std::min(d.nz, lz);
    } else {
        // longest z-segment that still gives every resident CTA several work items
        lz = d.nz;
        while (lz > 16 && (int64_t)tiles * ((d.nz + lz - 1) / lz) < 4LL * resident) lz = (lz + 1) / 2;
    }
    h->lz = lz;
    std::vector<uint32_t> word(h->n, 0);
    for (int64_t i = 0; i < h->n; ++i) word[i] = make_word(g.cls[i], g.payload[i], g.frozen[i] != 0, g.stencil[i] != 0);
    std::vector<int32_t> slot(tiles, -1);
    std::vector<char> skip(tiles, 0);
    int n_special = 0;
    for (int t = 0; t < tiles; ++t) {
        const int x0 = (t % h->tiles_x) * TILE_X, y0 = (t / h->tiles_x) * h->tile_y;
        bool special = false, all_frozen = true;
        for (int z = 0; z < d.nz; ++z)
            for (int y = y0; y < std::min(d.ny, y0 + h->tile_y); ++y)
                for (int x = x0; x < std::min(d.nx, x0 + TILE_X); ++x) {
                    const int64_t i = x + (int64_t)d.nx * (y + (int64_t)d.ny * z);
                    if (word[i]) special = true;
                    if (!g.frozen[i]) all_frozen = false;
                }
        if (all_frozen) skip[t] = 1;
        else if (special) slot[t] = n_special++;
    }
    h->n_special = n_special;

    // Non-bulk nodes of special tiles, in the order the step kernel exports their pulled
    // populations: slot, z, tile row, x.  Solid nodes of updated blocks need no populations:
    // the step kernel collides them in place; frozen nodes are never updated.  Neither is
    // in the list.
    std::vector<uint64_t> list_xyz;
    std::vector<uint32_t> list_word;
    std::vector<int32_t> row_base((size_t)n_special * d.nz * h->tile_y, 0);
    for (int t = 0; t < tiles; ++t) {
        if (slot[t] < 0) continue;
        const int x0 = (t % h->tiles_x) * TILE_X, y0 = (t / h->tiles_x) * h->tile_y;
        for (int z = 0; z < d.nz; ++z)
            for (int r = 0; r < h->tile_y; ++r) {
                row_base[((size_t)slot[t] * d.nz + z) * h->tile_y + r] = (int32_t)list_xyz.size();
                const int y = y0 + r;
                if (y >= d.ny) continue;
                for (int x = x0; x < std::min(d.nx, x0 + TILE_X); ++x) {
                    const int64_t i = x + (int64_t)d.nx * (y + (int64_t)d.ny * z);
                    const uint32_t wd = word[i];
                    // plain fluid nodes marked only as wall-stencil nodes are updated (and
                    // snapshotted) by the step kernel itself
                    if (wd == 0u || wd == NW_STENCIL || (wd & NW_FROZEN)) continue;
                    if ((wd & NW_CLASS_MASK) == C_SOLID) continue;
                    list_xyz.push_back((uint64_t)x | ((uint64_t)y << 21) | ((uint64_t)z << 42));
                    list_word.push_back(wd);
                }
            }
    }
    if (list_xyz.size() >= (size_t)INT32_MAX / 27)
        return fail(h, MRLBM_ERR_INVALID_ARG, "too many boundary nodes");
    h->n_list_pop = (int)list_xyz.size();
    h->n_list = h->n_list_pop;
    h->n_list_blocks = special_list_blocks(h->n_list);
    const int nseg = (d.nz + h->lz - 1) / h->lz;
    // work items are int32 `tile | segment << 20` (decoded in step_kernel)
    if (tiles > (1 << 20) || nseg > (1 << 11))
        return fail(h, MRLBM_ERR_INVALID_ARG,
                    "grid too large for the work-item encoding (at most 2^20 xy tiles and 2^11 z segments)");
    // tiles without boundary nodes go to the bulk variant of the step kernel, the others to
    // the variant that reads node words: two launches, each over its own items
    std::vector<int32_t> items, items_sp;
    for (int s = 0; s < nseg; ++s)
        for (int t = 0; t < tiles; ++t)
            if (!skip[t]) (slot[t] >= 0 ? items_sp : items).push_back(t | (s << 20));
    h->n_items = (int)items.size();
    h->n_items_sp = (int)items_sp.size();
    h->n_ctas = h->n_items ? std::max(1, std::min(h->n_items, resident)) : 0;
    h->n_ctas_sp = h->n_items_sp ? std::max(1, std::min(h->n_items_sp, resident)) : 0;
    h->h_items = items;
    h->h_items_sp = items_sp;
    items.insert(items.end(), items_sp.begin(), items_sp.end());

    if (h->d_word) {
        CK(h, upload(&h->d_tile_slot, slot.data(), slot.size()));
        if (n_special > 0) {
            const size_t side_floats = (size_t)n_special * d.nz * TILE_X * h->tile_y * 16;
            CK(h, cudaMalloc((void **)&h->d_side, side_floats * sizeof(float)));
            CK(h, cudaMemset(h->d_side, 0, side_floats * sizeof(float)));
        }
    }
    CK(h, upload(&h->d_items, items.data(), items.size()));
    CK(h, cudaMalloc((void **)&h->d_diag_part,
                     (size_t)(h->n_ctas + h->n_ctas_sp + h->n_list_blocks) * 2 * sizeof(double)));
    if (h->n_list > 0) {
        CK(h, upload(&h->d_list_xyz, list_xyz.data(), list_xyz.size()));
        CK(h, upload(&h->d_list_word, list_word.data(), list_word.size()));
        CK(h, upload(&h->d_row_base, row_base.data(), row_base.size()));
        if (h->n_list_pop > 0) CK(h, cudaMalloc((void **)&h->d_popbuf, (size_t)h->n_list_pop * 27 * sizeof(float)));
    }
    StepArgs &a = h->args;
    // a single case's items are uniform: CTAs stride through them, which keeps neighbouring
    // tiles in flight together (L2 reuse of the rim columns); batches claim items on demand
    a.work_counter = nullptr;
    a.items = h->d_items;
    a.n_items = h->n_items;
    a.tile_slot = h->d_tile_slot;
    a.side = h->d_side;
    a.list_xyz = h->d_list_xyz;
    a.list_word = h->d_list_word;
    a.n_list_pop = h->n_list_pop;
    a.n_list = h->n_list;
    a.popbuf = h->d_popbuf;
    a.row_base = h->d_row_base;
    a.tiles_x = h->tiles_x;
    a.tiles_y = h->tiles_y;
    a.tile_y = h->tile_y;
    a.lz = h->lz;
    CK(h, cudaMemcpy(h->d_args, &a, sizeof(StepArgs), cudaMemcpyHostToDevice));
    StepArgs asp = a;
    asp.items = h->d_items ? h->d_items + h->n_items : nullptr;
    asp.n_items = h->n_items_sp;
    asp.work_counter = nullptr;
    if (!h->d_args_sp) CK(h, cudaMalloc((void **)&h->d_args_sp, sizeof(StepArgs)));
    CK(h, cudaMemcpy(h->d_args_sp, &asp, sizeof(StepArgs), cudaMemcpyHostToDevice));
    return MRLBM_OK;
}

// One or more time steps of one handle: step kernel, node-list kernel, wall kernel and the
// sampled force / diagnostics reductions, all asynchronous on the handle's stream.
// The divergence flag as last copied back to the host (no synchronisation: the copy of a
// watchdog step lands in the pinned word while later steps are queued).
bool diverged_seen(const mrlbm_handle *h) {
    return h->h_status && (*(const volatile int *)h->h_status & kErrorDiverged);
}

int step_handle(mrlbm_handle *h, int32_t nsteps) {
    if (diverged_seen(h))
        return fail(h, MRLBM_ERR_DIVERGED, "the divergence watchdog found non-finite mass / energy sums");
    const int nb = (int)(h->geo.wall[0].list.size() + h->geo.wall[1].list.size());
    const int nbf = (int)(h->geo.wall[0].fluid_list.size() + h->geo.wall[1].fluid_list.size());
    for (int s = 0; s < nsteps; ++s) {
        const int64_t it = h->step;
        const bool fs = h->force_every > 0 && it % h->force_every == 0;
        const bool ds = h->diag_every > 0 && it % h->diag_every == 0;
        // watchdog steps compute the same sums as a sampled step, into their own slot
        const bool ws = !ds && h->watchdog_every > 0 && (it + 1) % h->watchdog_every == 0;
        StepLaunch L;
        L.ga = h->d_args;
        L.parity = h->parity;
        L.n_ctas = h->n_ctas;
        L.full_tiles = h->d.nx % TILE_X == 0 && h->d.ny % h->tile_y == 0;
        if (fs) {
            const int64_t slot = h->force_count % kRing;
            L.force = h->d_force_ring + slot * 10;
            CK(h, cudaMemsetAsync(L.force, 0, 10 * sizeof(double), h->stream));
            h->force_steps[slot] = it;
            ++h->force_count;
        }
        const bool sums = ds || ws;
        if (sums) L.diag_part = h->d_diag_part;
        const int n_step_parts = h->n_ctas + h->n_ctas_sp;
        // The boundary work of the step runs on the side stream, concurrently with the bulk
        // tiles: the boundary-tile step kernel, then the node-list kernel (it reads only the
        // populations that kernel exported) and the wall kernel (it reads only the list
        // kernel's stencil snapshots); their blocks fill the SMs the bulk launch leaves idle
        // in its last wave.  No bulk-tile node is read or written by them.
        cudaStream_t bs = h->stream;
        if (h->n_items_sp > 0) {
            StepLaunch Ls = L;
            Ls.ga = h->d_args_sp;
            Ls.n_ctas = h->n_ctas_sp;
            Ls.diag_part = sums ? h->d_diag_part + 2 * h->n_ctas : nullptr;
            CK(h, cudaEventRecord(h->ev_fork, h->stream));
            CK(h, cudaStreamWaitEvent(h->side_stream, h->ev_fork, 0));
            CK(h, launch_step(Ls, h->storage, h->tile_y, true, h->side_stream));
            bs = h->side_stream;
        }
        if (h->n_list > 0)
            CK(h, launch_special_list(L, h->storage, h->n_list_blocks, sums ? h->d_diag_part + 2 * n_step_parts : nullptr,
                                      bs));
        if (nb > 0) CK(h, launch_wall(L, h->storage, nb + (fs ? nbf : 0), bs));
        if (h->n_items_sp > 0) CK(h, cudaEventRecord(h->ev_join, h->side_stream));
        if (h->n_items > 0) CK(h, launch_step(L, h->storage, h->tile_y, false, h->stream));
        if (h->n_items_sp > 0) CK(h, cudaStreamWaitEvent(h->stream, h->ev_join, 0));
        if (h->ps_start >= 0 && it >= h->ps_start && it <= h->ps_end) {
            // statistics window: the post-step state (buffer parity ^ 1), as the reference's
            // post_process_step samples it
            ++h->ps_count;
            const int64_t slot = (h->ps_count - 1) % kRing;
            h->inlet_steps[(size_t)slot] = it;
            CK(h, launch_inlet_density(h->d_args, h->parity ^ 1, h->storage, h->d_inlet, (int)slot, h->ps_count,
                                       h->stream));
            for (int w = 0; w < h->geo.n_walls; ++w)
                CK(h, launch_surface_pressure(h->d_args, h->parity ^ 1, h->storage, w,
                                              (int)h->geo.wall[w].list.size(), h->d_ps_avg[w], h->ps_count,
                                              h->stream));
        }
        if (sums) {
            const int parts = n_step_parts + (h->n_list > 0 ? h->n_list_blocks : 0);
            if (ds) {
                const int64_t slot = h->diag_count % kRing;
                CK(h, launch_diag_finalize(h->d_diag_part, parts, h->d_diag_ring + slot * 2, h->d_error, h->stream));
                h->diag_steps[slot] = it;
                ++h->diag_count;
            } else {
                CK(h, launch_diag_finalize(h->d_diag_part, parts, h->d_watch, h->d_error, h->stream));
            }
            // the early refusal of mrlbm_step reads this copy: made at the watchdog's cadence only
            // (a step sampled in between adds no copy to the stream; mrlbm_sync reads the word
            // itself)
            if (h->watchdog_every > 0 && (it + 1) % h->watchdog_every == 0)
                CK(h, cudaMemcpyAsync(h->h_status, h->d_error, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        }
        if (h->d_sr_step) CK(h, launch_sr_tick(h->d_sr_step, h->stream));
        h->parity ^= 1;
        ++h->step;
    }
    return MRLBM_OK;
}

// Candidate z-segment lengths for the autotuner: 0 (the per-case heuristic) and powers of two
// below nz.
std::vector<int> lz_candidates(int nz) {
    std::vector<int> v{0};
    for (int lz = 8; lz < nz; lz *= 2) v.push_back(lz);
    return v;
}

// Saved time-step state: the current moment buffer and the step / sampling counters, so the
// autotuner's trial steps leave no trace.
struct SavedState {
    void *buf = nullptr;
    int parity = 0, force_every = 0, diag_every = 0;
    int64_t step = 0, force_count = 0, diag_count = 0;
    int64_t ps_start = -1, ps_end = -1;
};

int save_state(mrlbm_handle *h, SavedState &st) {
    // counters first: a failed save leaves them to restore_state unchanged
    st.parity = h->parity;
    st.force_every = h->force_every;
    st.diag_every = h->diag_every;
    st.step = h->step;
    st.force_count = h->force_count;
    st.diag_count = h->diag_count;
    st.ps_start = h->ps_start;
    st.ps_end = h->ps_end;
    const size_t bytes = (size_t)h->fs * h->vbytes;
    CK(h, cudaMalloc(&st.buf, bytes));
    CK(h, cudaMemcpyAsync(st.buf, h->m[h->parity], bytes, cudaMemcpyDeviceToDevice, h->stream));
    h->force_every = h->diag_every = 0;
    h->ps_start = h->ps_end = -1;  // no statistics-window samples from trial steps
    return MRLBM_OK;
}

// Put back what save_state kept (counters always; the field if it was saved) and free the copy.
int restore_state(mrlbm_handle *h, SavedState &st) {
    int rc = MRLBM_OK;
    if (st.buf) {
        const size_t bytes = (size_t)h->fs * h->vbytes;
        cudaError_t e = cudaMemcpyAsync(h->m[st.parity], st.buf, bytes, cudaMemcpyDeviceToDevice, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        cudaFree(st.buf);
        st.buf = nullptr;
        if (e != cudaSuccess) rc = cuda_fail(h, e, "restoring the saved field");
    }
    h->parity = st.parity;
    h->force_every = st.force_every;
    h->diag_every = st.diag_every;
    h->step = st.step;
    h->force_count = st.force_count;
    h->diag_count = st.diag_count;
    h->ps_start = st.ps_start;
    h->ps_end = st.ps_end;
    if (rc != MRLBM_OK) return rc;
    return sync_sr_step(h);
}

}  // namespace

extern "C" {

int mrlbm_abi_version(void) { return MRLBM_ABI_VERSION; }

const char *mrlbm_last_error(const mrlbm_handle *h) { return h ? h->err.c_str() : g_last_error.c_str(); }

int mrlbm_case_desc_default(mrlbm_case_desc *d, int32_t geometry) {
    if (!d) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null descriptor");
    std::memset(d, 0, sizeof(*d));
    d->struct_size = sizeof(*d);
    d->geometry = geometry;
    d->rho0 = 1.0f;
    d->triangular = 1;
    d->mass_bc = MRLBM_MASS_EQUILIBRIUM;
    d->bcf_mass_bc = MRLBM_MASS_EQUILIBRIUM;
    d->storage = MRLBM_STORAGE_F32;
    if (geometry == MRLBM_GEOM_CYLINDER) {
        // MRLBM_3D/src/cases/cylinder/constants.cuh:8-54
        const int D = 16, LW = 4 * D, LE = 16 * D, LN = 4 * D, LS = LN;
        d->nx = LW + D + LE;
        d->ny = LN + D + LS;
        d->nz = 3 * D;
        d->periodic[0] = 0;
        d->periodic[1] = 1;
        d->periodic[2] = 1;
        d->convective_outlet = 1;
        d->u_max = 0.1f;
        d->re = 100.0f;
        d->d_wall[0] = (float)D;
        d->xc = (float)(LW + 0.5 * (D - 1));
        d->yc = (float)(LS + 0.5 * (D - 1));
        d->scan_box[0] = LW - 4;
        d->scan_box[1] = LW + D + 4;
        d->scan_box[2] = LS - 4;
        d->scan_box[3] = LS + D + 4;
    } else if (geometry == MRLBM_GEOM_ANNULUS) {
        // MRLBM_3D/src/cases/annulus/constants.cuh:19-84
        const float d_out = 128.0f, r_out = 0.5f * d_out, r_in = 0.5f * r_out;
        d->nx = 136;
        d->ny = 136;
        d->nz = 256;
        d->periodic[0] = 0;
        d->periodic[1] = 0;
        d->periodic[2] = 1;
        d->u_max = 0.03f;
        d->re = 70.0f;
        d->d_wall[0] = 2.0f * r_in;
        d->d_wall[1] = d_out;
        d->xc = (float)(0.5 * (136 - 1));
        d->yc = (float)(0.5 * (136 - 1));
        const float vel_scale = d->u_max / r_in;
        d->wall_u[0][1] = vel_scale * r_in;
        d->scan_box[0] = 0;
        d->scan_box[1] = d->nx;
        d->scan_box[2] = 0;
        d->scan_box[3] = d->ny;
    } else if (geometry == MRLBM_GEOM_NONE) {
        d->nx = d->ny = d->nz = 64;
        d->periodic[0] = d->periodic[1] = d->periodic[2] = 1;
        d->u_max = 0.05f;
        d->re = 1600.0f;
        d->length = (float)(64.0 / (2.0 * M_PI));
    } else {
        return fail(nullptr, MRLBM_ERR_INVALID_ARG, "unknown geometry");
    }
    return MRLBM_OK;
}

int mrlbm_case_desc_finalize(mrlbm_case_desc *d) {
    if (!d || d->struct_size != sizeof(*d)) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "descriptor size mismatch");
    if (d->nx <= 0 || d->ny <= 0 || d->nz <= 0 || d->nx % 8 || d->ny % 8 || d->nz % 4)
        return fail(nullptr, MRLBM_ERR_INVALID_ARG, "grid must be positive multiples of 8 x 8 x 4");
    if (d->nx < 8 || d->ny < 8 || d->nz < 4) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "grid too small");
    if ((int64_t)d->nx * d->ny * d->nz >= (1LL << 31) * 8)
        return fail(nullptr, MRLBM_ERR_INVALID_ARG, "grid too large");
    if (d->storage < 0 || d->storage > 3) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "bad storage");
    if (d->geometry < 0 || d->geometry > 2) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "bad geometry");
    if (!(d->rho0 > 0.f)) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "rho0 must be positive");
    if (d->omega <= 0.f && !(d->re > 0.f)) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "need re > 0 or omega > 0");
    if (d->geometry == MRLBM_GEOM_NONE && d->omega <= 0.f && !(d->length > 0.f))
        return fail(nullptr, MRLBM_ERR_INVALID_ARG, "need length > 0 to derive omega");
    if (d->geometry == MRLBM_GEOM_ANNULUS && !(d->d_wall[1] > d->d_wall[0]))
        return fail(nullptr, MRLBM_ERR_INVALID_ARG, "annulus needs d_wall[1] > d_wall[0]");
    if (d->scan_box[0] == 0 && d->scan_box[1] == 0 && d->scan_box[2] == 0 && d->scan_box[3] == 0) {
        // classification window left unset: derive it the way the reference's constants do
        // (nodeClass.cuh:174-177, LW-4 .. LW+D+4 with LW = XC - (D-1)/2; the whole plane for
        // the annulus, annulus/nodeClass.cuh:311-315), clipped to the grid
        if (d->geometry == MRLBM_GEOM_CYLINDER) {
            const int dd = (int)std::ceil(d->d_wall[0]);
            const int lw = (int)std::floor(d->xc - 0.5f * (d->d_wall[0] - 1.0f));
            const int ls = (int)std::floor(d->yc - 0.5f * (d->d_wall[0] - 1.0f));
            d->scan_box[0] = std::max(0, lw - 4);
            d->scan_box[1] = std::min(d->nx, lw + dd + 4);
            d->scan_box[2] = std::max(0, ls - 4);
            d->scan_box[3] = std::min(d->ny, ls + dd + 4);
        } else {
            d->scan_box[1] = d->nx;
            d->scan_box[3] = d->ny;
        }
    }
    Derived der;
    const std::string e = derive(*d, der);
    if (!e.empty()) return fail(nullptr, MRLBM_ERR_INVALID_ARG, e);
    return MRLBM_OK;
}

int mrlbm_create_host(const mrlbm_case_desc *din, mrlbm_handle **out) {
    if (!din || !out) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    mrlbm_case_desc d = *din;
    int rc = mrlbm_case_desc_finalize(&d);
    if (rc) return rc;
    std::unique_ptr<mrlbm_handle> h(new mrlbm_handle());
    h->d = d;
    derive(h->d, h->der);
    const std::string ge = classify(h->d, h->geo);
    if (!ge.empty()) return fail(nullptr, MRLBM_ERR_INVALID_ARG, ge);
    h->n = (int64_t)d.nx * d.ny * d.nz;
    h->storage = d.storage;
    h->vbytes = storage_element_bytes(d.storage);
    h->host_only = true;
    *out = h.release();
    return MRLBM_OK;
}

int mrlbm_create(const mrlbm_case_desc *din, mrlbm_handle **out) {
    if (!din || !out) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    mrlbm_case_desc d = *din;
    int rc = mrlbm_case_desc_finalize(&d);
    if (rc) return rc;
    std::unique_ptr<mrlbm_handle> h(new mrlbm_handle());
    h->d = d;
    derive(h->d, h->der);
    CK(h.get(), cudaGetDevice(&h->dev));
    CK(h.get(), cudaDeviceGetAttribute(&h->n_sm, cudaDevAttrMultiProcessorCount, h->dev));
    int major = 0, minor = 0;
    CK(h.get(), cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, h->dev));
    CK(h.get(), cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, h->dev));
    if (!(major == 10 && minor == 3)) {
        fail(nullptr, MRLBM_ERR_UNSUPPORTED, "libmrlbm is built for sm_103a (GB300) only");
        return MRLBM_ERR_UNSUPPORTED;
    }
    CK(h.get(), cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking));
    h->stream = h->own_stream;
    CK(h.get(), cudaStreamCreateWithFlags(&h->side_stream, cudaStreamNonBlocking));
    CK(h.get(), cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming));
    CK(h.get(), cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));

    // geometry on the host
    const std::string ge = classify(h->d, h->geo);
    if (!ge.empty()) {
        const std::string msg = ge;
        free_all(h.get());
        return fail(nullptr, MRLBM_ERR_INVALID_ARG, msg);
    }
    const Geometry &g = h->geo;
    h->n = (int64_t)d.nx * d.ny * d.nz;
    // storage elements per moment buffer (the hybrid mode keeps 7 words per node)
    h->fs = aos_elements(d.nx, d.ny, d.nz, d.storage == MRLBM_STORAGE_F16_U32 ? 7 : 10);
    h->storage = d.storage;
    h->vbytes = storage_element_bytes(d.storage);
    for (int k = 0; k < 3; ++k) {
        float s = d.storage_scale[k];
        if (d.storage == MRLBM_STORAGE_F32 || (d.storage == MRLBM_STORAGE_F16_U32 && k == 1)) s = 1.f;  // FP32 values
        else if (!(s > 0.f)) {
            const float u = d.u_max > 0.f ? d.u_max : 0.05f;
            s = k == 1 ? 1.0f / u : 1.0f / (u * u);
        }
        h->sc.s[k] = s;
        h->sc.is[k] = 1.0f / s;
    }

    // node words (tile independent)
    std::vector<uint32_t> word(h->n, 0);
    bool any_special = false;
    int64_t n_fluid = 0;
    for (int64_t i = 0; i < h->n; ++i) {
        word[i] = make_word(g.cls[i], g.payload[i], g.frozen[i] != 0, g.stencil[i] != 0);
        if (word[i]) any_special = true;
        const uint32_t c = g.cls[i];
        if (!g.frozen[i] && c != C_SOLID && c != C_INNER && c != C_OUTER) ++n_fluid;
    }
    h->n_fluid = n_fluid;

    mrlbm_handle *H = h.get();
    const size_t mbytes = (size_t)h->fs * h->vbytes;
    CK(H, cudaMalloc(&h->m[0], mbytes));
    CK(H, cudaMalloc(&h->m[1], mbytes));
    CK(H, cudaMemset(h->m[0], 0, mbytes));
    CK(H, cudaMemset(h->m[1], 0, mbytes));
    if (any_special) CK(H, upload(&h->d_word, word.data(), word.size()));
    for (int w = 0; w < g.n_walls; ++w) {
        const WallData &wd = g.wall[w];
        CK(H, upload(&h->d_wf[w][0], wd.nx.data(), wd.nx.size()));
        CK(H, upload(&h->d_wf[w][1], wd.ny.data(), wd.ny.size()));
        CK(H, upload(&h->d_wf[w][2], wd.delta.data(), wd.delta.size()));
        CK(H, upload(&h->d_wm[w][0], wd.in_mask.data(), wd.in_mask.size()));
        CK(H, upload(&h->d_wm[w][1], wd.out_mask.data(), wd.out_mask.size()));
        CK(H, upload(&h->d_wl[w][0], wd.list.data(), wd.list.size()));
        CK(H, upload(&h->d_wl[w][1], wd.fluid_list.data(), wd.fluid_list.size()));
    }
    {
        std::vector<uint32_t> tags(512);
        std::memcpy(tags.data(), g.tag_in_mask, 256 * 4);
        std::memcpy(tags.data() + 256, g.tag_out_mask, 256 * 4);
        CK(H, upload(&h->d_tag, tags.data(), tags.size()));
    }
    CK(H, cudaMalloc((void **)&h->d_error, sizeof(int)));
    CK(H, cudaMemset(h->d_error, 0, sizeof(int)));
    CK(H, cudaMalloc((void **)&h->d_watch, 2 * sizeof(double)));
    CK(H, cudaHostAlloc((void **)&h->h_status, sizeof(int), cudaHostAllocDefault));
    *h->h_status = 0;
    h->watchdog_every = d.watchdog_every == 0 ? kWatchdogDefault : (d.watchdog_every < 0 ? 0 : d.watchdog_every);
    CK(H, cudaMalloc((void **)&h->d_force_ring, (size_t)kRing * 10 * sizeof(double)));
    CK(H, cudaMalloc((void **)&h->d_diag_ring, (size_t)kRing * 2 * sizeof(double)));
    h->force_steps.assign(kRing, -1);
    h->diag_steps.assign(kRing, -1);

    StepArgs &a = h->args;
    a.m[0] = h->m[0];
    a.m[1] = h->m[1];
    a.nxb = (d.nx + kXBlock - 1) / kXBlock;
    a.word = h->d_word;
    a.nx = d.nx;
    a.ny = d.ny;
    a.nz = d.nz;
    a.omega = h->der.omega;
    a.rho0 = d.rho0;
    a.u_max = d.u_max;
    a.convective = d.convective_outlet;
    a.current_update = d.neumann_current_update;
    a.bcf_strong = d.bcf_mass_bc == MRLBM_MASS_STRONG;
    a.wall_strong = d.mass_bc == MRLBM_MASS_STRONG;
    a.xc = d.xc;
    a.yc = d.yc;
    a.sc = h->sc;
    for (int w = 0; w < g.n_walls; ++w) {
        WallArgs &W = a.wall[w];
        W.nx = h->d_wf[w][0];
        W.ny = h->d_wf[w][1];
        W.delta = h->d_wf[w][2];
        W.in_mask = h->d_wm[w][0];
        W.out_mask = h->d_wm[w][1];
        W.list = h->d_wl[w][0];
        W.fluid_list = h->d_wl[w][1];
        W.nb = (int)g.wall[w].list.size();
        W.nbf = (int)g.wall[w].fluid_list.size();
        W.r_wall = 0.5f * d.d_wall[w];
        W.dir = w == 1 ? -1.0f : 1.0f;
        for (int k = 0; k < 3; ++k) W.u_wall[k] = d.wall_u[w][k];
    }
    a.tag_in = h->d_tag;
    a.tag_out = h->d_tag ? h->d_tag + 256 : nullptr;
    a.error = h->d_error;
    if (d.stochastic_rounding && d.storage != MRLBM_STORAGE_F32) {
        CK(H, cudaMalloc((void **)&h->d_sr_step, sizeof(uint32_t)));
        CK(H, cudaMemset(h->d_sr_step, 0, sizeof(uint32_t)));
        a.sr_step = h->d_sr_step;
    }
    CK(H, cudaMalloc((void **)&h->d_args, sizeof(StepArgs)));
    {
        int ty = 16, lz = 0;
        default_tiling(ty, lz);
        const int rc = setup_tiling(H, ty, lz);
        if (rc != MRLBM_OK) return rc;
    }
    CK(H, cudaDeviceSynchronize());
    *out = h.release();
    return MRLBM_OK;
}

int mrlbm_destroy(mrlbm_handle *h) {
    if (!h) return MRLBM_OK;
    if (h->batch) return fail(h, MRLBM_ERR_STATE, "this handle belongs to a batch: use mrlbm_batch_destroy");
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (!h->host_only) free_all(h);
    delete h;
    return MRLBM_OK;
}

int mrlbm_set_stream(mrlbm_handle *h, void *cuda_stream) {
    if (!h) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null handle");
    if (h->host_only) return fail(h, MRLBM_ERR_STATE, "host-only handle has no device state");
    if (h->batch) return fail(h, MRLBM_ERR_STATE, "this handle belongs to a batch: it runs on the batch stream");
    CK(h, cudaStreamSynchronize(h->stream));
    h->stream = cuda_stream ? (cudaStream_t)cuda_stream : h->own_stream;
    return MRLBM_OK;
}

int mrlbm_get_info(const mrlbm_handle *h, mrlbm_info *info) {
    if (!h || !info) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null argument");
    std::memset(info, 0, sizeof(*info));
    info->nx = h->d.nx;
    info->ny = h->d.ny;
    info->nz = h->d.nz;
    info->n_nodes = h->n;
    for (int w = 0; w < 2; ++w) {
        info->nb[w] = (int32_t)h->geo.wall[w].list.size();
        info->nb_fluid[w] = (int32_t)h->geo.wall[w].fluid_list.size();
        info->nb_solid[w] = (int32_t)h->geo.wall[w].solid_list.size();
    }
    info->omega = h->der.omega;
    info->tau = h->der.tau;
    info->step = h->step;
    info->storage = h->storage;
    info->bytes_per_value = h->vbytes;
    info->n_active_items = h->n_items + h->n_items_sp;
    info->tile[0] = TILE_X;
    info->tile[1] = h->tile_y;
    info->tile[2] = h->lz;
    info->reserved[0] = h->n_ctas + h->n_ctas_sp;
    info->reserved[1] = h->n_special;
    info->reserved[2] = (int32_t)std::min<int64_t>(h->n_fluid, INT32_MAX);
    return MRLBM_OK;
}

int mrlbm_init(mrlbm_handle *h, int32_t kind, const double *params, int32_t n_params) {
    if (!h) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null handle");
    if (h->host_only) return fail(h, MRLBM_ERR_STATE, "host-only handle has no device state");
    if (kind < 0 || kind > MRLBM_INIT_NOISY_UNIFORM) return fail(h, MRLBM_ERR_INVALID_ARG, "bad init kind");
    InitArgs ia;
    ia.m_a = h->m[0];
    ia.m_b = h->m[1];
    ia.nx = h->d.nx;
    ia.ny = h->d.ny;
    ia.nz = h->d.nz;
    ia.kind = kind;
    ia.rho0 = h->d.rho0;
    ia.u_max = h->d.u_max;
    ia.sc = h->sc;
    const int need = kind == MRLBM_INIT_TAYLOR_GREEN ? 2 : kind == MRLBM_INIT_UNIFORM ? 3
                     : kind == MRLBM_INIT_NOISY_UNIFORM ? 5 : 0;
    if (n_params < need || (need && !params)) return fail(h, MRLBM_ERR_INVALID_ARG, "missing init parameters");
    for (int k = 0; k < need && k < 8; ++k) ia.p[k] = params[k];
    if (int rc = clear_divergence(h)) return rc;
    CK(h, launch_init(ia, h->storage, h->stream));
    h->parity = 0;
    h->step = 0;
    h->force_count = h->diag_count = 0;
    std::fill(h->force_steps.begin(), h->force_steps.end(), -1);
    std::fill(h->diag_steps.begin(), h->diag_steps.end(), -1);
    h->initialized = true;
    return sync_sr_step(h);
}

int mrlbm_set_sampling(mrlbm_handle *h, int32_t force_every, int32_t diag_every) {
    if (!h) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null handle");
    if (force_every < 0 || diag_every < 0) return fail(h, MRLBM_ERR_INVALID_ARG, "negative sampling period");
    h->force_every = h->geo.n_walls ? force_every : 0;
    h->diag_every = diag_every;
    return MRLBM_OK;
}

int mrlbm_step(mrlbm_handle *h, int32_t nsteps) {
    if (!h) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null handle");
    if (h->host_only) return fail(h, MRLBM_ERR_STATE, "host-only handle has no device state");
    if (h->batch) return fail(h, MRLBM_ERR_STATE, "this handle belongs to a batch: step it with mrlbm_batch_step");
    if (!h->initialized) return fail(h, MRLBM_ERR_STATE, "mrlbm_init / mrlbm_set_moments must come first");
    if (nsteps < 0) return fail(h, MRLBM_ERR_INVALID_ARG, "negative step count");
    return step_handle(h, nsteps);
}

// Test hook for the autotuners' failure paths: MRLBM_FAULT_AUTOTUNE_TRIAL=k makes trial k
// (1-based) of every autotune call fail as a CUDA error would, on the host, before it launches.
static int injected_trial_failure(int trial) {
    const char *v = std::getenv("MRLBM_FAULT_AUTOTUNE_TRIAL");
    return v && std::atoi(v) == trial;
}

int mrlbm_autotune(mrlbm_handle *h, int32_t trial_steps, int32_t tile_out[3]) {
    if (!h) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null handle");
    if (h->host_only) return fail(h, MRLBM_ERR_STATE, "host-only handle has no device state");
    if (h->batch) return fail(h, MRLBM_ERR_STATE, "this handle belongs to a batch: use mrlbm_batch_autotune");
    if (trial_steps < 1) return fail(h, MRLBM_ERR_INVALID_ARG, "need at least one trial step");
    SavedState st;
    int rc = save_state(h, st);
    if (rc) {
        if (st.buf) cudaFree(st.buf);
        return rc;
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const int ty0 = h->tile_y, lz0 = h->lz;
    float best = 1e30f;
    int best_ty = ty0, best_lz = lz0;
    // the trials; any failure leaves the loop with its status and falls through to the
    // clean-up below, which always runs
    auto trials = [&]() -> int {
        CK(h, cudaEventCreate(&e0));
        CK(h, cudaEventCreate(&e1));
        int trial = 0, r;
        for (int ty : {4, 8, 16}) {
            for (int lz : lz_candidates(h->d.nz)) {
                if (injected_trial_failure(++trial))
                    return fail(h, MRLBM_ERR_CUDA, "autotune trial " + std::to_string(trial) + ": injected failure");
                if ((r = setup_tiling(h, ty, lz)) != MRLBM_OK) return r;
                if ((r = step_handle(h, 1)) != MRLBM_OK) return r;  // warm-up
                CK(h, cudaEventRecord(e0, h->stream));
                if ((r = step_handle(h, trial_steps)) != MRLBM_OK) return r;
                CK(h, cudaEventRecord(e1, h->stream));
                CK(h, cudaEventSynchronize(e1));
                float ms = 0.f;
                CK(h, cudaEventElapsedTime(&ms, e0, e1));
                if (ms < best) {
                    best = ms;
                    best_ty = ty;
                    best_lz = h->lz;
                }
            }
        }
        return MRLBM_OK;
    };
    rc = trials();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    // keep the fastest tiling, or the one in use before a failed search; then the saved state
    std::string first_err = rc != MRLBM_OK ? h->err : std::string();
    int r2 = setup_tiling(h, rc == MRLBM_OK ? best_ty : ty0, rc == MRLBM_OK ? best_lz : lz0);
    int r3 = restore_state(h, st);
    if (st.buf) cudaFree(st.buf);
    if (rc != MRLBM_OK) return fail(h, rc, first_err);
    if (r2 != MRLBM_OK) return r2;
    if (r3 != MRLBM_OK) return r3;
    if (tile_out) {
        tile_out[0] = TILE_X;
        tile_out[1] = h->tile_y;
        tile_out[2] = h->lz;
    }
    return MRLBM_OK;
}

int mrlbm_sync(mrlbm_handle *h) {
    if (!h) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null handle");
    if (h->host_only) return fail(h, MRLBM_ERR_STATE, "host-only handle has no device state");
    CK(h, cudaStreamSynchronize(h->stream));
    int e = 0;
    CK(h, cudaMemcpy(&e, h->d_error, sizeof(int), cudaMemcpyDeviceToHost));
    *h->h_status = e;
    if (e & ~kErrorDiverged)
        return fail(h, MRLBM_ERR_CUDA, "device reported a stencil lookup failure (code " + std::to_string(e) + ")");
    if (e & kErrorDiverged)
        return fail(h, MRLBM_ERR_DIVERGED, "the divergence watchdog found non-finite mass / energy sums");
    if (h->diag_count > 0) {
        double v[2];
        const int64_t slot = (h->diag_count - 1) % kRing;
        CK(h, cudaMemcpy(v, h->d_diag_ring + slot * 2, sizeof(v), cudaMemcpyDeviceToHost));
        if (!std::isfinite(v[0]) || !std::isfinite(v[1]))
            return fail(h, MRLBM_ERR_DIVERGED, "mass / energy diagnostics are not finite");
    }
    return MRLBM_OK;
}

int mrlbm_get_moments(mrlbm_handle *h, uint32_t mask, int32_t layout, float *host, size_t count) {
    if (!h || !host) return fail(h, MRLBM_ERR_INVALID_ARG, "null argument");
    if (h->host_only) return fail(h, MRLBM_ERR_STATE, "host-only handle has no device state");
    if (!h->initialized) return fail(h, MRLBM_ERR_STATE, "no state yet");
    mask &= MRLBM_FIELD_ALL;
    const int nf = __builtin_popcount(mask);
    if (nf == 0 || count < (size_t)nf * h->n) return fail(h, MRLBM_ERR_INVALID_ARG, "host buffer too small");
    if (layout != MRLBM_LAYOUT_LEXICOGRAPHIC && layout != MRLBM_LAYOUT_REF_TILED)
        return fail(h, MRLBM_ERR_INVALID_ARG, "bad layout");
    const void *src = h->m[h->parity];
    int rc = ensure_stage(h, (size_t)nf * h->n * 4);
    if (rc) return rc;
    CK(h, launch_convert(src, nullptr, nullptr, h->d_stage, mask, layout, h->d.nx, h->d.ny, h->d.nz, h->storage, h->sc,
                         0, h->stream));
    CK(h, cudaMemcpyAsync(host, h->d_stage, (size_t)nf * h->n * 4, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return MRLBM_OK;
}

int mrlbm_set_moments(mrlbm_handle *h, uint32_t mask, int32_t layout, const float *host, size_t count) {
    if (!h || !host) return fail(h, MRLBM_ERR_INVALID_ARG, "null argument");
    if (h->host_only) return fail(h, MRLBM_ERR_STATE, "host-only handle has no device state");
    mask &= MRLBM_FIELD_ALL;
    const int nf = __builtin_popcount(mask);
    if (nf == 0 || count < (size_t)nf * h->n) return fail(h, MRLBM_ERR_INVALID_ARG, "host buffer too small");
    if (!h->initialized && mask != MRLBM_FIELD_ALL)
        return fail(h, MRLBM_ERR_STATE, "the first mrlbm_set_moments must set every field");
    if (layout != MRLBM_LAYOUT_LEXICOGRAPHIC && layout != MRLBM_LAYOUT_REF_TILED)
        return fail(h, MRLBM_ERR_INVALID_ARG, "bad layout");
    void *cur = h->m[h->parity], *oth = h->m[h->parity ^ 1];
    int rc = ensure_stage(h, (size_t)nf * h->n * 4);
    if (rc) return rc;
    if ((rc = clear_divergence(h)) != MRLBM_OK) return rc;
    CK(h, cudaMemcpyAsync(h->d_stage, host, (size_t)nf * h->n * 4, cudaMemcpyHostToDevice, h->stream));
    CK(h, launch_convert(nullptr, cur, oth, h->d_stage, mask, layout, h->d.nx, h->d.ny, h->d.nz, h->storage, h->sc, 1,
                         h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    h->initialized = true;
    return MRLBM_OK;
}

int mrlbm_get_node_types(mrlbm_handle *h, int32_t layout, uint32_t *host, size_t count) {
    if (!h || !host) return fail(h, MRLBM_ERR_INVALID_ARG, "null argument");
    if (count < (size_t)h->n) return fail(h, MRLBM_ERR_INVALID_ARG, "host buffer too small");
    for (int64_t i = 0; i < h->n; ++i)
        host[node_index_for_layout(h, i, layout)] = ((uint32_t)h->geo.cls[i] << 20) | (h->geo.payload[i] & 0xFFFFFu);
    return MRLBM_OK;
}

int mrlbm_get_boundary(mrlbm_handle *h, int32_t wall, int32_t what, int32_t layout, void *host, size_t count) {
    if (!h || !host || wall < 0 || wall > 1) return fail(h, MRLBM_ERR_INVALID_ARG, "bad argument");
    const WallData &wd = h->geo.wall[wall];
    auto copy_list = [&](const std::vector<int64_t> &v) -> int {
        if (count < v.size()) return fail(h, MRLBM_ERR_INVALID_ARG, "host buffer too small");
        int64_t *o = (int64_t *)host;
        for (size_t i = 0; i < v.size(); ++i) o[i] = node_index_for_layout(h, v[i], layout);
        return MRLBM_OK;
    };
    auto copy_f = [&](const std::vector<float> &v) -> int {
        if (count < v.size()) return fail(h, MRLBM_ERR_INVALID_ARG, "host buffer too small");
        std::memcpy(host, v.data(), v.size() * 4);
        return MRLBM_OK;
    };
    auto copy_u = [&](const uint32_t *v, size_t n) -> int {
        if (count < n) return fail(h, MRLBM_ERR_INVALID_ARG, "host buffer too small");
        std::memcpy(host, v, n * 4);
        return MRLBM_OK;
    };
    switch (what) {
        case MRLBM_BND_LIST: return copy_list(wd.list);
        case MRLBM_BND_NORMAL_X: return copy_f(wd.nx);
        case MRLBM_BND_NORMAL_Y: return copy_f(wd.ny);
        case MRLBM_BND_DELTA: return copy_f(wd.delta);
        case MRLBM_BND_IN_MASK: return copy_u(wd.in_mask.data(), wd.in_mask.size());
        case MRLBM_BND_OUT_MASK: return copy_u(wd.out_mask.data(), wd.out_mask.size());
        case MRLBM_BND_FLUID_LIST: return copy_list(wd.fluid_list);
        case MRLBM_BND_TAG_IN_MASK: return copy_u(h->geo.tag_in_mask, 256);
        case MRLBM_BND_TAG_OUT_MASK: return copy_u(h->geo.tag_out_mask, 256);
        case MRLBM_BND_SOLID_LIST: return copy_list(wd.solid_list);
        default: return fail(h, MRLBM_ERR_INVALID_ARG, "bad boundary array id");
    }
}

int mrlbm_get_forces(mrlbm_handle *h, int64_t step, double out[10]) {
    if (!h || !out) return fail(h, MRLBM_ERR_INVALID_ARG, "null argument");
    if (h->host_only) return fail(h, MRLBM_ERR_STATE, "host-only handle has no device state");
    CK(h, cudaStreamSynchronize(h->stream));
    const int64_t lo = std::max<int64_t>(0, h->force_count - kRing);
    for (int64_t c = h->force_count - 1; c >= lo; --c) {
        const int64_t slot = c % kRing;
        if (step < 0 || h->force_steps[slot] == step) {
            CK(h, cudaMemcpy(out, h->d_force_ring + slot * 10, 10 * sizeof(double), cudaMemcpyDeviceToHost));
            return MRLBM_OK;
        }
    }
    return fail(h, MRLBM_ERR_STATE, "no force sample for that step");
}

int mrlbm_get_force_history(mrlbm_handle *h, int32_t max_steps, int64_t *steps, double *forces, int32_t *n_out) {
    if (!h || !n_out || max_steps < 0) return fail(h, MRLBM_ERR_INVALID_ARG, "bad argument");
    if (h->host_only) return fail(h, MRLBM_ERR_STATE, "host-only handle has no device state");
    CK(h, cudaStreamSynchronize(h->stream));
    const int64_t avail = std::min<int64_t>(h->force_count, kRing);
    const int64_t n = std::min<int64_t>(avail, max_steps);
    std::vector<double> ring((size_t)kRing * 10);
    if (n > 0) CK(h, cudaMemcpy(ring.data(), h->d_force_ring, ring.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int64_t k = 0; k < n; ++k) {
        const int64_t c = h->force_count - n + k;
        const int64_t slot = c % kRing;
        if (steps) steps[k] = h->force_steps[slot];
        if (forces) std::memcpy(forces + k * 10, ring.data() + slot * 10, 10 * sizeof(double));
    }
    *n_out = (int32_t)n;
    return MRLBM_OK;
}

int mrlbm_get_diagnostics(mrlbm_handle *h, int32_t max_steps, int64_t *steps, double *values, int32_t *n_out) {
    if (!h || !n_out || max_steps < 0) return fail(h, MRLBM_ERR_INVALID_ARG, "bad argument");
    if (h->host_only) return fail(h, MRLBM_ERR_STATE, "host-only handle has no device state");
    CK(h, cudaStreamSynchronize(h->stream));
    const int64_t avail = std::min<int64_t>(h->diag_count, kRing);
    const int64_t n = std::min<int64_t>(avail, max_steps);
    for (int64_t k = 0; k < n; ++k) {
        const int64_t c = h->diag_count - n + k;
        const int64_t slot = c % kRing;
        double v[2];
        CK(h, cudaMemcpy(v, h->d_diag_ring + slot * 2, sizeof(v), cudaMemcpyDeviceToHost));
        if (steps) steps[k] = h->diag_steps[slot];
        if (values) {
            values[2 * k + 0] = (double)h->n_fluid * h->d.rho0 + v[0];
            values[2 * k + 1] = v[1];
        }
    }
    *n_out = (int32_t)n;
    return MRLBM_OK;
}

int mrlbm_step_periodic_noalloc(const float *m_in, float *m_out, int32_t nx, int32_t ny, int32_t nz, float omega,
                                float rho0, double *diag, void *cuda_stream) {
    NoAllocStep p;
    p.m_in = m_in;
    p.m_out = m_out;
    p.nx = nx;
    p.ny = ny;
    p.nz = nz;
    p.omega = omega;
    p.rho0 = rho0;
    p.diag_host = diag;
    p.stream = (cudaStream_t)cuda_stream;
    std::string err;
    const int rc = noalloc_periodic_step(p, err);
    if (rc != MRLBM_OK) return fail(nullptr, rc, err);
    return MRLBM_OK;
}

}  // extern "C"

// ---- batches of independent cases (no counterpart in the reference) -------------------------

namespace {

int bfail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

#define BCK(call)                                                                  \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) return bfail(MRLBM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

void batch_free_graphs(mrlbm_batch *b) {
    for (auto &row : b->graph)
        for (auto &g : row) {
            if (g) cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

void batch_free_tables(mrlbm_batch *b) {
    batch_free_graphs(b);
    for (void **p : {(void **)&b->d_cases, (void **)&b->d_items, (void **)&b->d_list_blocks,
                     (void **)&b->d_wall_blocks, (void **)&b->d_ring, (void **)&b->d_slot, (void **)&b->d_ba,
                     (void **)&b->d_ba_sp, (void **)&b->d_work}) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
}

// Tile every case with (ty, lz) and rebuild the merged work-item and block tables.
int batch_set_tiling(mrlbm_batch *b, int ty, int lz) {
    BCK(cudaStreamSynchronize(b->stream));
    for (mrlbm_handle *h : b->h) {
        const int rc = setup_tiling(h, ty, lz);
        if (rc != MRLBM_OK) return rc;
    }
    batch_free_tables(b);
    b->tile_y = ty;
    b->lz = lz;
    const int n = (int)b->h.size();
    std::vector<const StepArgs *> cases(n);
    std::vector<double *> ring(n);
    std::vector<int2> items, items_sp;
    std::vector<int4> lblocks, wblocks;
    for (int c = 0; c < n; ++c) {
        mrlbm_handle *h = b->h[c];
        cases[c] = h->d_args;
        ring[c] = h->d_force_ring;
        for (int32_t it : h->h_items) items.push_back(make_int2(c, it));
        for (int32_t it : h->h_items_sp) items_sp.push_back(make_int2(c, it));
        if (h->n_list > 0) {
            const int first = (int)lblocks.size();
            for (int k = 0; k < h->n_list_blocks; ++k) lblocks.push_back(make_int4(c, first, h->n_list_blocks, 0));
        }
        const int nw = (int)(h->geo.wall[0].list.size() + h->geo.wall[1].list.size() +
                             h->geo.wall[0].fluid_list.size() + h->geo.wall[1].fluid_list.size());
        if (nw > 0) {
            const int first = (int)wblocks.size(), nblk = (nw + 127) / 128;
            for (int k = 0; k < nblk; ++k) wblocks.push_back(make_int4(c, first, nblk, 0));
        }
    }
    b->n_items = (int)items.size();
    b->n_items_sp = (int)items_sp.size();
    items.insert(items.end(), items_sp.begin(), items_sp.end());
    b->n_list_blocks = (int)lblocks.size();
    b->n_wall_blocks = (int)wblocks.size();
    int per_sm = step_kernel_max_ctas_per_sm(b->storage, ty);
    if (per_sm <= 0) per_sm = 1;
    b->n_ctas = b->n_items ? std::max(1, std::min(b->n_items, per_sm * b->h[0]->n_sm)) : 0;
    b->n_ctas_sp = b->n_items_sp ? std::max(1, std::min(b->n_items_sp, per_sm * b->h[0]->n_sm)) : 0;
    auto up = [&](auto **dptr, const auto &v) -> cudaError_t {
        using T = typename std::remove_reference<decltype(v)>::type::value_type;
        if (v.empty()) return cudaSuccess;
        cudaError_t e = cudaMalloc((void **)dptr, v.size() * sizeof(T));
        if (e != cudaSuccess) return e;
        return cudaMemcpy((void *)*dptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    };
    BCK(up(&b->d_cases, cases));
    BCK(up(&b->d_ring, ring));
    BCK(up(&b->d_items, items));
    BCK(up(&b->d_list_blocks, lblocks));
    BCK(up(&b->d_wall_blocks, wblocks));
    BCK(cudaMalloc((void **)&b->d_slot, sizeof(int)));
    BCK(cudaMemset(b->d_slot, 0, sizeof(int)));
    BCK(cudaMalloc((void **)&b->d_work, 2 * sizeof(int)));
    BCK(cudaMemset(b->d_work, 0, 2 * sizeof(int)));
    BatchArgs ba;
    ba.work_counter = b->d_work;
    ba.cases = b->d_cases;
    ba.items = b->d_items;
    ba.n_items = b->n_items;
    ba.list_blocks = b->d_list_blocks;
    ba.wall_blocks = b->d_wall_blocks;
    ba.force_ring = b->d_ring;
    ba.force_slot = b->d_slot;
    BCK(cudaMalloc((void **)&b->d_ba, sizeof(BatchArgs)));
    BCK(cudaMemcpy(b->d_ba, &ba, sizeof(BatchArgs), cudaMemcpyHostToDevice));
    BatchArgs bsp = ba;
    bsp.items = b->d_items ? b->d_items + b->n_items : nullptr;
    bsp.n_items = b->n_items_sp;
    bsp.work_counter = b->d_work + 1;
    BCK(cudaMalloc((void **)&b->d_ba_sp, sizeof(BatchArgs)));
    BCK(cudaMemcpy(b->d_ba_sp, &bsp, sizeof(BatchArgs), cudaMemcpyHostToDevice));
    BCK(prepare_step_batch(b->storage, ty));  // both variants, before any capture
    return MRLBM_OK;
}

// The three batched launches of one step.
int batch_launch(mrlbm_batch *b, int parity, int force) {
    BCK(cudaMemsetAsync(b->d_work, 0, 2 * sizeof(int), b->stream));
    if (b->n_items_sp > 0) {
        BCK(cudaEventRecord(b->ev_fork, b->stream));
        BCK(cudaStreamWaitEvent(b->side_stream, b->ev_fork, 0));
        BCK(launch_step_batch(b->d_ba_sp, parity, b->storage, b->tile_y, true, b->n_ctas_sp, b->side_stream));
        BCK(cudaEventRecord(b->ev_join, b->side_stream));
    }
    if (b->n_items > 0) BCK(launch_step_batch(b->d_ba, parity, b->storage, b->tile_y, false, b->n_ctas, b->stream));
    if (b->n_items_sp > 0) BCK(cudaStreamWaitEvent(b->stream, b->ev_join, 0));
    BCK(launch_special_list_batch(b->d_ba, parity, force, b->storage, b->n_list_blocks, b->stream));
    BCK(launch_wall_batch(b->d_ba, parity, force, b->storage, b->n_wall_blocks, b->stream));
    bool any_sr = false;
    for (const mrlbm_handle *h : b->h) any_sr = any_sr || h->d_sr_step != nullptr;
    if (any_sr) BCK(launch_sr_tick_cases(b->d_cases, (int)b->h.size(), b->stream));
    return MRLBM_OK;
}

int batch_graph(mrlbm_batch *b, int parity, int force, cudaGraphExec_t *out) {
    if (!b->graph[parity][force]) {
        cudaGraph_t g = nullptr;
        BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = batch_launch(b, parity, force);
        const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
        if (rc != MRLBM_OK) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        BCK(ce);
        const cudaError_t ie = cudaGraphInstantiate(&b->graph[parity][force], g, 0);
        cudaGraphDestroy(g);
        BCK(ie);
    }
    *out = b->graph[parity][force];
    return MRLBM_OK;
}

// Advance every case one step with the batched kernels (graph replay or direct launches).
int batch_step_once(mrlbm_batch *b, bool use_graph) {
    const int64_t it = b->step;
    const int force = b->force_every > 0 && it % b->force_every == 0;
    if (force) {
        const int64_t slot = b->force_count % kRing;
        BCK(launch_batch_force_begin(b->d_ring, (int)b->h.size(), (int)slot, b->d_slot, b->stream));
        for (mrlbm_handle *h : b->h) {
            if (!h->geo.n_walls) continue;  // as mrlbm_set_sampling: no walls, no force samples
            h->force_steps[slot] = it;
            ++h->force_count;
        }
        ++b->force_count;
    }
    if (use_graph) {
        cudaGraphExec_t g = nullptr;
        const int rc = batch_graph(b, b->parity, force, &g);
        if (rc != MRLBM_OK) return rc;
        BCK(cudaGraphLaunch(g, b->stream));
    } else {
        const int rc = batch_launch(b, b->parity, force);
        if (rc != MRLBM_OK) return rc;
    }
    b->parity ^= 1;
    ++b->step;
    for (mrlbm_handle *h : b->h) {
        h->parity = b->parity;
        h->step = b->step;
    }
    return MRLBM_OK;
}

int batch_check(mrlbm_batch *b) {
    if (!b) return bfail(MRLBM_ERR_INVALID_ARG, "null batch");
    for (mrlbm_handle *h : b->h)
        if (!h->initialized) return bfail(MRLBM_ERR_STATE, "initialise every case of the batch first");
    return MRLBM_OK;
}

}  // namespace

extern "C" {

int mrlbm_batch_create(const mrlbm_case_desc *descs, int32_t n, mrlbm_batch **out) {
    if (!descs || !out || n <= 0) return bfail(MRLBM_ERR_INVALID_ARG, "need descriptors and n > 0");
    *out = nullptr;
    std::unique_ptr<mrlbm_batch> b(new mrlbm_batch());
    auto cleanup = [&]() {
        for (mrlbm_handle *h : b->h) {
            h->batch = nullptr;
            h->stream = h->own_stream;
            mrlbm_destroy(h);
        }
        b->h.clear();
        if (b->stream) cudaStreamDestroy(b->stream);
    };
    for (int i = 0; i < n; ++i) {
        mrlbm_handle *h = nullptr;
        const int rc = mrlbm_create(&descs[i], &h);
        if (rc != MRLBM_OK) {
            const std::string msg = "case " + std::to_string(i) + ": " + g_last_error;
            cleanup();
            return bfail(rc, msg);
        }
        b->h.push_back(h);
        if (h->storage != b->h[0]->storage) {
            cleanup();
            return bfail(MRLBM_ERR_INVALID_ARG, "all cases of a batch must use the same moment storage");
        }
    }
    b->storage = b->h[0]->storage;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->side_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        cleanup();
        return bfail(MRLBM_ERR_CUDA, "cannot create the batch stream");
    }
    for (mrlbm_handle *h : b->h) {
        cudaStreamSynchronize(h->stream);
        h->stream = b->stream;
        h->batch = b.get();
    }
    int ty = 16, lz = 0;
    default_tiling(ty, lz);
    const int rc = batch_set_tiling(b.get(), ty, lz);
    if (rc != MRLBM_OK) {
        const std::string msg = g_last_error;
        batch_free_tables(b.get());
        cleanup();
        return bfail(rc, msg);
    }
    *out = b.release();
    return MRLBM_OK;
}

int mrlbm_batch_destroy(mrlbm_batch *b) {
    if (!b) return MRLBM_OK;
    cudaStreamSynchronize(b->stream);
    batch_free_tables(b);
    for (mrlbm_handle *h : b->h) {
        h->batch = nullptr;
        h->stream = h->own_stream;
        mrlbm_destroy(h);
    }
    if (b->stream) cudaStreamDestroy(b->stream);
    if (b->side_stream) cudaStreamDestroy(b->side_stream);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_join) cudaEventDestroy(b->ev_join);
    delete b;
    return MRLBM_OK;
}

int mrlbm_batch_size(const mrlbm_batch *b) { return b ? (int)b->h.size() : 0; }

int mrlbm_batch_handle(mrlbm_batch *b, int32_t i, mrlbm_handle **out) {
    if (!b || !out || i < 0 || i >= (int)b->h.size()) return bfail(MRLBM_ERR_INVALID_ARG, "bad batch index");
    *out = b->h[i];
    return MRLBM_OK;
}

int mrlbm_batch_set_sampling(mrlbm_batch *b, int32_t force_every) {
    if (!b || force_every < 0) return bfail(MRLBM_ERR_INVALID_ARG, "bad batch sampling");
    b->force_every = force_every;
    for (mrlbm_handle *h : b->h) {
        h->force_every = h->geo.n_walls ? force_every : 0;
        h->diag_every = 0;
    }
    return MRLBM_OK;
}

int mrlbm_batch_step(mrlbm_batch *b, int32_t nsteps) {
    int rc = batch_check(b);
    if (rc != MRLBM_OK) return rc;
    if (nsteps < 0) return bfail(MRLBM_ERR_INVALID_ARG, "negative step count");
    for (int s = 0; s < nsteps; ++s)
        if ((rc = batch_step_once(b, true)) != MRLBM_OK) return rc;
    return MRLBM_OK;
}

int mrlbm_batch_step_sequential(mrlbm_batch *b, int32_t nsteps) {
    int rc = batch_check(b);
    if (rc != MRLBM_OK) return rc;
    if (nsteps < 0) return bfail(MRLBM_ERR_INVALID_ARG, "negative step count");
    for (int s = 0; s < nsteps; ++s) {
        for (mrlbm_handle *h : b->h)
            if ((rc = step_handle(h, 1)) != MRLBM_OK) return bfail(rc, g_last_error);
        if (b->force_every > 0 && b->step % b->force_every == 0) ++b->force_count;
        b->parity ^= 1;
        ++b->step;
    }
    return MRLBM_OK;
}

int mrlbm_batch_sync(mrlbm_batch *b) {
    if (!b) return bfail(MRLBM_ERR_INVALID_ARG, "null batch");
    BCK(cudaStreamSynchronize(b->stream));
    for (mrlbm_handle *h : b->h) {
        const int rc = mrlbm_sync(h);
        if (rc != MRLBM_OK) return rc;
    }
    return MRLBM_OK;
}

int mrlbm_batch_autotune(mrlbm_batch *b, int32_t trial_steps, int32_t tile_out[3]) {
    int rc = batch_check(b);
    if (rc != MRLBM_OK) return rc;
    if (trial_steps < 1) return bfail(MRLBM_ERR_INVALID_ARG, "need at least one trial step");
    BCK(cudaStreamSynchronize(b->stream));
    std::vector<SavedState> saved(b->h.size());
    auto release = [&]() {
        for (SavedState &st : saved)
            if (st.buf) {
                cudaFree(st.buf);
                st.buf = nullptr;
            }
    };
    for (size_t c = 0; c < b->h.size(); ++c)
        if ((rc = save_state(b->h[c], saved[c])) != MRLBM_OK) {
            // cases saved so far get their sampling back; nothing has stepped yet
            for (size_t k = 0; k <= c; ++k) restore_state(b->h[k], saved[k]);
            release();
            return rc;
        }
    const int saved_parity = b->parity, saved_force = b->force_every;
    const int64_t saved_step = b->step;
    const int ty0 = b->tile_y, lz0 = b->lz;
    b->force_every = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int max_nz = 0;
    for (mrlbm_handle *h : b->h) max_nz = std::max(max_nz, h->d.nz);
    float best = 1e30f;
    int best_ty = ty0, best_lz = lz0;
    auto trials = [&]() -> int {
        BCK(cudaEventCreate(&e0));
        BCK(cudaEventCreate(&e1));
        int trial = 0, r;
        for (int ty : {4, 8, 16}) {
            for (int lz : lz_candidates(max_nz)) {
                if (injected_trial_failure(++trial))
                    return bfail(MRLBM_ERR_CUDA, "batch autotune trial " + std::to_string(trial) + ": injected failure");
                if ((r = batch_set_tiling(b, ty, lz)) != MRLBM_OK) return r;
                if ((r = batch_step_once(b, false)) != MRLBM_OK) return r;  // warm-up
                BCK(cudaEventRecord(e0, b->stream));
                for (int s = 0; s < trial_steps; ++s)
                    if ((r = batch_step_once(b, false)) != MRLBM_OK) return r;
                BCK(cudaEventRecord(e1, b->stream));
                BCK(cudaEventSynchronize(e1));
                float ms = 0.f;
                BCK(cudaEventElapsedTime(&ms, e0, e1));
                if (ms < best) {
                    best = ms;
                    best_ty = ty;
                    best_lz = lz;
                }
            }
        }
        return MRLBM_OK;
    };
    rc = trials();
    const std::string first_err = rc != MRLBM_OK ? mrlbm::g_last_error : std::string();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaStreamSynchronize(b->stream);
    int r2 = batch_set_tiling(b, rc == MRLBM_OK ? best_ty : ty0, rc == MRLBM_OK ? best_lz : lz0);
    int r3 = MRLBM_OK;
    for (size_t c = 0; c < b->h.size(); ++c) {
        const int r = restore_state(b->h[c], saved[c]);
        if (r != MRLBM_OK && r3 == MRLBM_OK) r3 = r;
    }
    release();
    b->parity = saved_parity;
    b->step = saved_step;
    b->force_every = saved_force;
    if (rc != MRLBM_OK) return bfail(rc, first_err);
    if (r2 != MRLBM_OK) return r2;
    if (r3 != MRLBM_OK) return r3;
    if (tile_out) {
        tile_out[0] = TILE_X;
        tile_out[1] = b->tile_y;
        tile_out[2] = b->lz;
    }
    return MRLBM_OK;
}

}  // extern "C"
