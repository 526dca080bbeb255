/*
 * mrlbm.h — C ABI of the GB300-native D3Q27 moment-representation LBM (MR-LBM) solver.
 *
 * One handle = one simulation case (grid, physics, curved-wall geometry) living in the
 * HBM of the current CUDA device, advanced by hand-written sm_103a kernels.  Plain C
 * types only: no torch or CUDA types appear in the signatures (the optional stream is
 * passed as an opaque pointer).  Every entry point returns an int status (MRLBM_OK = 0,
 * negative on error) and never exits the process; mrlbm_last_error() holds the message.
 *
 * Reference interfaces replaced (paths inside sakthi-lbm/MRLBM_3D_CUDA):
 *   - the compile-time case constants   MRLBM_3D/src/cases/cylinder/constants.cuh:8-54,
 *                                       MRLBM_3D/src/cases/annulus/constants.cuh:8-84,
 *                                       MRLBM_3D/src/config.h:8       -> mrlbm_case_desc
 *   - the case plugin table `struct Case` MRLBM_3D/src/common/globalStructs.cuh:46-62 and
 *     setup_case                        MRLBM_3D/src/solve_mrlbm.cu:3-24 -> mrlbm_create
 *   - initialize_simulation             MRLBM_3D/src/simulation.cu:13-35 -> mrlbm_create + mrlbm_init
 *   - the time loop streaming / boundary_treatment / collision
 *                                       MRLBM_3D/src/main.cu:21-35   -> mrlbm_step
 *   - copyMomentsDeviceToHost / HostToDevice
 *                                       MRLBM_3D/src/solve_mrlbm.cuh:113-160 -> mrlbm_get/set_moments
 *   - cylinder_incoming/outgoing_force_kernal + write_forces
 *                                       MRLBM_3D/src/cases/cylinder/cylinder_kernels.cu:181-236,
 *                                       MRLBM_3D/src/statistics/stat_header.cuh:16-33 -> mrlbm_get_forces
 *   - write_checkpoint / read_checkpoint MRLBM_3D/src/restart/restart_io.cu:3-36 -> mrlbm_checkpoint_*
 *   - write_vti_3d                      MRLBM_3D/src/output/saveData.cu:42-116 -> mrlbm_write_vti
 *   - checkCudaErrors (exit on error)   MRLBM_3D/src/utils/cudaHelpers.cuh:10-21 -> status codes
 */
#ifndef MRLBM_H
#define MRLBM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MRLBM_ABI_VERSION 1

/* ---- status codes ---------------------------------------------------------------- */
#define MRLBM_OK 0
#define MRLBM_ERR_INVALID_ARG (-1) /* bad descriptor / argument (also the tau / Mach guards) */
#define MRLBM_ERR_CUDA (-2)        /* a CUDA runtime call failed                              */
#define MRLBM_ERR_DIVERGED (-3)    /* NaN / Inf seen by the mass watchdog                     */
#define MRLBM_ERR_TIMEOUT (-4)     /* a bounded device wait gave up                          */
#define MRLBM_ERR_IO (-5)          /* file could not be read / written                        */
#define MRLBM_ERR_UNSUPPORTED (-6) /* option not built (e.g. device has no sm_103a)           */
#define MRLBM_ERR_STATE (-7)       /* call out of order (e.g. step before init)               */
#define MRLBM_ERR_NOMEM (-8)       /* device allocation failed                                */

/* ---- enumerations -------------------------------------------------------------------- */
#define MRLBM_GEOM_NONE 0     /* no solid: periodic box or plain channel                  */
#define MRLBM_GEOM_CYLINDER 1 /* circular cylinder, axis along z (cases/cylinder)          */
#define MRLBM_GEOM_ANNULUS 2  /* two concentric cylinders, axis along z (cases/annulus)     */

#define MRLBM_STORAGE_F32 0  /* moments stored as float                                   */
#define MRLBM_STORAGE_F16 1  /* moments stored as IEEE half, scaled deviations            */
#define MRLBM_STORAGE_BF16 2 /* moments stored as bfloat16, scaled deviations             */
#define MRLBM_STORAGE_F16_U32 3 /* velocity in FP32, rho - rho0 and m as FP16 scaled deviations */

#define MRLBM_MASS_EQUILIBRIUM 0 /* MassBC::Equilibrium (common/types.cuh:14-19)           */
#define MRLBM_MASS_STRONG 1      /* MassBC::Strong                                         */

#define MRLBM_INIT_REFERENCE_NOISE 0 /* the reference's initializer, bit for bit:
                                        solver/initializeLBM.cu:39-121 (rho0, u = (0, 0,
                                        1e-4 U sin(2 pi z / NZ) + hash noise), m_ij = 0)       */
#define MRLBM_INIT_REST 1            /* rho = rho0, u = 0, m = 0                              */
#define MRLBM_INIT_TAYLOR_GREEN 2    /* params[0] = u0, params[1] = L (wavelength / 2 pi)     */
#define MRLBM_INIT_UNIFORM 3         /* params[0..2] = (ux, uy, uz), rho = rho0, m = u u      */
#define MRLBM_INIT_NOISY_UNIFORM 4   /* params[0..2] = u, params[3] = rel. amplitude,
                                        params[4] = seed: u (1 + a xi), xi ~ U(-1, 1) hashed   */

#define MRLBM_LAYOUT_LEXICOGRAPHIC 0 /* idx = x + NX (y + NY z)                               */
#define MRLBM_LAYOUT_REF_TILED 1     /* the reference's IDX_BLOCK 8x8x4 tiles (core/index.cuh:11-28) */

/* Moment fields, in the order of the reference's checkpoint (restart/restart_io.cu:38-52).
 * RHO is stored as rho - rho0, exactly like nodeVar::rho. */
#define MRLBM_NFIELDS 10
#define MRLBM_FIELD_RHO (1u << 0)
#define MRLBM_FIELD_UX (1u << 1)
#define MRLBM_FIELD_UY (1u << 2)
#define MRLBM_FIELD_UZ (1u << 3)
#define MRLBM_FIELD_MXX (1u << 4)
#define MRLBM_FIELD_MYY (1u << 5)
#define MRLBM_FIELD_MZZ (1u << 6)
#define MRLBM_FIELD_MXY (1u << 7)
#define MRLBM_FIELD_MXZ (1u << 8)
#define MRLBM_FIELD_MYZ (1u << 9)
#define MRLBM_FIELD_ALL 0x3FFu

/* Boundary arrays readable with mrlbm_get_boundary (wall 0 = inner / cylinder, 1 = outer). */
#define MRLBM_BND_LIST 0        /* int64  [NB]  node index, layout given by the call          */
#define MRLBM_BND_NORMAL_X 1    /* float  [NB]  unit_nx (cylinder_helpers.cuh:10-47)         */
#define MRLBM_BND_NORMAL_Y 2    /* float  [NB]  unit_ny                                      */
#define MRLBM_BND_DELTA 3       /* float  [NB]  wall distance delta_w                        */
#define MRLBM_BND_IN_MASK 4     /* uint32 [NB]  incomingMask (cylinder_helpers.cuh:134-228)  */
#define MRLBM_BND_OUT_MASK 5    /* uint32 [NB]  outgoingMask                                 */
#define MRLBM_BND_FLUID_LIST 6  /* int64  [NB_FLUID] BCFLUID node index                       */
#define MRLBM_BND_TAG_IN_MASK 7 /* uint32 [256] d_incomingMask_bcfluid (cylinder_helpers.cuh:230-299) */
#define MRLBM_BND_TAG_OUT_MASK 8 /* uint32 [256] d_outgoingMask_bcfluid                       */
#define MRLBM_BND_SOLID_LIST 9  /* int64  [NB_SOLID] BCSOLID node index (z walls only,     
                                   cylinder_helpers.cuh:49-114 bcsolidList)                  */

/* ---- case descriptor -------------------------------------------------------------------
 * A runtime POD replacing the reference's per-case constexpr headers.  Fill it with
 * mrlbm_case_desc_default(), edit, then mrlbm_create().  omega <= 0 means "derive it the
 * way the reference does" (nu = U L / Re in float, tau = 0.5 + 3 nu, omega = 1 / tau). */
typedef struct mrlbm_case_desc {
    uint32_t struct_size; /* = sizeof(mrlbm_case_desc)                                  */
    int32_t geometry;     /* MRLBM_GEOM_*                                               */
    int32_t nx, ny, nz;   /* lattice size; multiples of 8, 8 and 4 (initializeLBM.cuh:60-62) */
    int32_t periodic[3];  /* X_PERIODIC, Y_PERIODIC, Z_PERIODIC                          */
    float u_max;          /* U_MAX: inlet / characteristic velocity                      */
    float rho0;           /* RHO_0                                                       */
    float re;             /* RE                                                          */
    float length;         /* L of nu = U L / Re for GEOM_NONE (cylinder uses D, annulus the gap) */
    float omega;          /* 1 / tau; <= 0: derived                                      */
    /* curved walls */
    float xc, yc;         /* XC, YC: axis of the cylinder(s)                             */
    float d_wall[2];      /* D_WALL (cylinder) / D_IN, D_OUT (annulus)                    */
    float wall_u[2][3];   /* UXP/UYP/UZP_INNER and _OUTER: wall velocity in the frame
                             rotated to the local normal (curvedLBM.cu:93-101)            */
    int32_t scan_box[4];  /* x0, x1, y0, y1: window of the node classification scans
                             (nodeClass.cuh:174-177: LW-4 .. LW+D+4, LS-4 .. LS+D+4);
                             all 0: mrlbm_case_desc_finalize derives it from xc, yc, d_wall */
    int32_t triangular;   /* 1: triangular (BCFLUID) classification, 0: staircase         */
    int32_t mass_bc;      /* MASS_CONSERV for the curved wall: MRLBM_MASS_*              */
    int32_t bcf_mass_bc;  /* BCF_MASS_CONSERV for BCFLUID nodes                          */
    int32_t convective_outlet;      /* CONVECTIVE_OUTLET (east face blend with |u_x|)   */
    int32_t neumann_current_update; /* NEUMANN_CURRENT_UPDATE (outlet uses streamed pops) */
    /* storage */
    int32_t storage;      /* MRLBM_STORAGE_*                                             */
    float storage_scale[3]; /* low-precision storage scales for (rho - rho0, u, m); 0 = auto */
    int32_t stochastic_rounding; /* FP16 / BF16 only: 1 rounds the time-step stores
                                    stochastically (hardware cvt.rs with hashed random bits
                                    per node, field pair and step) instead of to nearest     */
    int32_t watchdog_every; /* divergence watchdog period in steps, independent of sampling:
                               every this many steps the step computes its FP64 mass / energy
                               sums on the device and flags non-finite ones, and mrlbm_step /
                               mrlbm_sync return MRLBM_ERR_DIVERGED once the flag is seen;
                               0: the default (64), < 0: off                               */
    int32_t reserved[14];
} mrlbm_case_desc;

typedef struct mrlbm_info {
    int32_t nx, ny, nz;
    int64_t n_nodes;
    int32_t nb[2];        /* curved boundary nodes per wall (NODE_INNER / NODE_OUTER)     */
    int32_t nb_fluid[2];  /* BCFLUID nodes per wall                                      */
    float omega, tau;
    int64_t step;         /* steps taken since init                                       */
    int32_t storage;
    int32_t bytes_per_value;
    int32_t n_active_items;  /* work items (tile column x z-segment) the step kernel visits */
    int32_t tile[3];      /* tile x, tile y, z-segment length used by the step kernel     */
    int32_t nb_solid[2];  /* BCSOLID nodes per wall (z walls only)                       */
    int32_t reserved[6];
} mrlbm_info;

typedef struct mrlbm_handle mrlbm_handle;
typedef struct mrlbm_batch mrlbm_batch;

/* ---- lifecycle ------------------------------------------------------------------------- */
int mrlbm_abi_version(void);
/* Fill *d with the reference's shipped constants for `geometry` (cylinder: 336x144x48,
 * D = 16, Re = 100, U = 0.1; annulus: 136x136x256, r = 32 / 64, Re = 70, U = 0.03; none:
 * 64^3 periodic box). */
int mrlbm_case_desc_default(mrlbm_case_desc *d, int32_t geometry);
/* Validate and derive omega (tau / Mach guards of initializeLBM.cuh:8-26 as error codes). */
int mrlbm_case_desc_finalize(mrlbm_case_desc *d);
int mrlbm_create(const mrlbm_case_desc *d, mrlbm_handle **out);
/* Host-only handle: node classification, boundary lists and info, no device memory (no
 * GPU needed).  Device calls on it return MRLBM_ERR_STATE. */
int mrlbm_create_host(const mrlbm_case_desc *d, mrlbm_handle **out);
int mrlbm_destroy(mrlbm_handle *h);
const char *mrlbm_last_error(const mrlbm_handle *h); /* h == NULL: last error of this thread */
/* Launch on `cuda_stream` (a cudaStream_t) instead of the handle's own stream; NULL restores it. */
int mrlbm_set_stream(mrlbm_handle *h, void *cuda_stream);
int mrlbm_get_info(const mrlbm_handle *h, mrlbm_info *info);

/* ---- time stepping ----------------------------------------------------------------------- */
int mrlbm_init(mrlbm_handle *h, int32_t init_kind, const double *params, int32_t n_params);
/* Advance n steps (stream + boundary + collide per step), asynchronously on the stream. */
int mrlbm_step(mrlbm_handle *h, int32_t nsteps);
/* Force sampling every `force_every` steps (0 = off), mass / energy every `diag_every`. */
int mrlbm_set_sampling(mrlbm_handle *h, int32_t force_every, int32_t diag_every);
int mrlbm_sync(mrlbm_handle *h);

/* ---- field access (FP32 on the host, any storage on the device) --------------------------- */
int mrlbm_get_moments(mrlbm_handle *h, uint32_t field_mask, int32_t layout, float *host, size_t count);
int mrlbm_set_moments(mrlbm_handle *h, uint32_t field_mask, int32_t layout, const float *host, size_t count);
/* Node types in the reference encoding (type << 20 | index, common/nodeTypeMap.cuh:76-96). */
int mrlbm_get_node_types(mrlbm_handle *h, int32_t layout, uint32_t *host, size_t count);
int mrlbm_get_boundary(mrlbm_handle *h, int32_t wall, int32_t what, int32_t layout, void *host, size_t count);

/* ---- statistics ------------------------------------------------------------------------------
 * Per sampled step and wall: Fx, Fy, Fz, mass flux, torque_z about (xc, yc), accumulated in
 * FP64 (statistics/forces.cu:25-133 sums them in float).  out[w*5 + k]. */
int mrlbm_get_forces(mrlbm_handle *h, int64_t step, double out[10]);
/* Up to max_steps most recent samples: steps[i], forces[i*10 + w*5 + k]. */
int mrlbm_get_force_history(mrlbm_handle *h, int32_t max_steps, int64_t *steps, double *forces, int32_t *n_out);
/* Mass sum(rho) and kinetic energy 0.5 sum(|u|^2) over non-solid nodes, FP64, per sampled step. */
int mrlbm_get_diagnostics(mrlbm_handle *h, int32_t max_steps, int64_t *steps, double *values, int32_t *n_out);

/* ---- files in the reference formats --------------------------------------------------------- */
/* restart.bin (restart/restart_io.cu:3-92): int32 step count, the 10 moment arrays (rho - rho0
 * first) in the tiled IDX_BLOCK order, then the six face-population arrays of its 8 x 8 x 4
 * blocks (rebuilt here from the moments, which is what they hold after a reference step).
 * Loading takes the moments and the step count; the face arrays carry no other state. */
int mrlbm_checkpoint_save(mrlbm_handle *h, const char *path);
int mrlbm_checkpoint_load(mrlbm_handle *h, const char *path);
/* data<10000000+it>.vti (output/saveData.cu:42-231): rho, ux, uy, uz with NaN velocity on
 * solid nodes; annulus cases write rho, uz, u_theta, u_radial (velocities / u_max). */
int mrlbm_write_vti(mrlbm_handle *h, const char *path);
/* master.pvd listing data<10000000+it>.vti for it = 0, macr_save, ... <= max_iter
 * (output/saveData.cu:3-40). */
int mrlbm_write_master_pvd(const char *path, int32_t macr_save, int32_t max_iter);
/* forces.dat `iter Fx Fy Fz` and mass_flux.dat `iter m` of wall `wall`, %.16f
 * (statistics/stat_header.cuh:16-51); either path may be NULL.  append = 0 rewrites the
 * files from every sample still in the device ring, append = 1 adds the samples taken since
 * the previous call. */
int mrlbm_write_forces(mrlbm_handle *h, int32_t wall, const char *forces_path, const char *mass_path, int32_t append);
/* Statistics window: steps start..end (inclusive; start < 0 switches it off).  After each step
 * in it, like cylinder_post_process (cases/cylinder/cylinder_kernels.cu:147-175), the
 * time-averaged wall pressure (compute_surface_pressure, :238-283) and the inlet density
 * (compute_inlet_average_density, :285-338) are sampled; set before stepping, it restarts both
 * averages. */
int mrlbm_set_pressure_window(mrlbm_handle *h, int64_t start, int64_t end);
/* pressure.dat `theta z Cp` rows per wall node (cases/cylinder/cylinder_kernels.cuh:251-285). */
int mrlbm_write_pressure(mrlbm_handle *h, int32_t wall, const char *path);
/* inlet_density.dat `iter rho_in rho_in_average`, %.16f (statistics/stat_header.cuh:53-72):
 * mean density of the x = 0 face per window step and the running mean of the samples before
 * it (the reference writes the line before it updates the mean).  append as for
 * mrlbm_write_forces. */
int mrlbm_write_inlet_density(mrlbm_handle *h, const char *path, int32_t append);
/* The node lists of the grid_layout directory for the z = 0 slice, `x y z type index` per line, into the
 * directory `dir` (write_geometry_files, cases/cylinder/cylinder_helpers.cuh:388-470):
 * inner, outer, bcfluid_inner, bcfluid_outer, bcsolid_inner, bcsolid_outer, solid, fluid,
 * others.  Host only; works on host-only handles. */
int mrlbm_write_geometry(const mrlbm_handle *h, const char *dir);

/* ---- allocation-free step (no counterpart in the reference) ------------------------------------
 * One time step of a fully periodic box (no walls, no inlet / outlet) from m_in to m_out,
 * for callers that cannot allocate device memory: it calls no cudaMalloc / cudaFree and no
 * allocating library routine.  The step kernel's scratch (argument block, work items,
 * diagnostics partials) is one fixed 64 KiB array in the library's device image, which
 * bounds the grid to at most 11776 xy tiles of 32 x 16 nodes (ceil(nx/32) * ceil(ny/16)),
 * e.g. 2048 x 2944 nodes per z plane; larger grids are rejected with MRLBM_ERR_INVALID_ARG.
 * Every call shares that array and it keeps the last call's contents (each call rewrites
 * what it reads and clears its error word); calls that overlap on the GPU (two streams or
 * two host threads) race on it.
 * m_in / m_out: device pointers, 16-byte aligned, not overlapping, FP32 moments in the
 * solver's storage layout: field f of node (x, y, z) at element
 * (((z*ny + y)*ceil(nx/32) + x/32)*10 + f)*32 + x%32, fields in the order of
 * MRLBM_FIELD_* with field 0 holding rho - rho0; nz*ny*ceil(nx/32)*320 floats each.
 * Grid: positive multiples of 8 x 8 x 4.  diag: NULL, or {mass, kinetic energy} as
 * mrlbm_get_diagnostics, in which case the call waits for the step.  Otherwise it is
 * asynchronous on `cuda_stream` (a cudaStream_t; NULL = default stream). */
int mrlbm_step_periodic_noalloc(const float *m_in, float *m_out, int32_t nx, int32_t ny, int32_t nz, float omega,
                                float rho0, double *diag, void *cuda_stream);

/* ---- autotuning and batches (no counterpart in the reference: its tile shape is a
 * compile-time constant and it runs one case per process) ----------------------------------- */
/* Time every tile height (4, 8, 16) with every z-segment length (the built-in heuristic and
 * powers of two below nz) over `trial_steps` steps and keep the fastest.  The moments, step
 * counter and sampling state are restored afterwards; results do not depend on the tiling.
 * tile_out (optional): {32, tile height, z-segment length}. */
int mrlbm_autotune(mrlbm_handle *h, int32_t trial_steps, int32_t tile_out[3]);
/* Several independent cases (uneven grids allowed; one moment storage for all) advanced
 * together: per step one persistent step-kernel launch over the work items of every case,
 * one node-list launch and one wall launch, replayed from CUDA graphs.  Proposed in place of
 * running the reference once per case (MRLBM_3D/src/main.cu:7-40). */
int mrlbm_batch_create(const mrlbm_case_desc *descs, int32_t n, mrlbm_batch **out);
int mrlbm_batch_destroy(mrlbm_batch *b);
int mrlbm_batch_size(const mrlbm_batch *b);
/* Handle of case i, for init / set / get moments, forces and info.  It runs on the batch's
 * stream; mrlbm_step, mrlbm_destroy, mrlbm_set_stream and mrlbm_autotune on it return
 * MRLBM_ERR_STATE. */
int mrlbm_batch_handle(mrlbm_batch *b, int32_t i, mrlbm_handle **h);
/* Force sampling period for every case (0 = off); batches keep no mass / energy samples. */
int mrlbm_batch_set_sampling(mrlbm_batch *b, int32_t force_every);
int mrlbm_batch_step(mrlbm_batch *b, int32_t nsteps);
/* The same steps as plain per-case launches, case after case (the unbatched comparison). */
int mrlbm_batch_step_sequential(mrlbm_batch *b, int32_t nsteps);
/* Batch-wide tile height and z-segment cap, timed like mrlbm_autotune. */
int mrlbm_batch_autotune(mrlbm_batch *b, int32_t trial_steps, int32_t tile_out[3]);
int mrlbm_batch_sync(mrlbm_batch *b);

#ifdef __cplusplus
}
#endif
#endif /* MRLBM_H */
