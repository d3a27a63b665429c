/*
 * lbffs_cuda.h -- C ABI of the GB300 lattice-Boltzmann step for LBFFS.
 *
 * This header is the drop-in boundary for the OpenCL section of LBFFS's driver
 * (D3Q19_opencl/ns.cpp:382-603, D3Q27_opencl/ns.cpp): one context replaces the
 * cl::Context / cl::CommandQueue / 27 cl::Buffer objects / 4 KernelFunctors, and
 * the host keeps computing everything else (input.hpp, setBoundaryConditions.hpp,
 * walls.hpp, stl.hpp, initialization.hpp, restart.hpp, write.hpp) unchanged.
 *
 * Conventions
 *  - Every call returns an int status: LBFFS_OK (0) or a negative LBFFS_E_* code.
 *    lbffs_last_error() returns a message for the last failing call on a context
 *    (or on the calling thread when the context pointer is NULL).  No C++
 *    exception crosses the boundary.
 *  - Arrays use the reference's layout: cell index ic = nx*ny*k + nx*j + i
 *    (src/base.hpp:20), populations f[q*E + ic] with E = nx*ny*nz
 *    (src/base.hpp:30), the reference's velocity order (D3Q19.hpp:14-27).
 *  - Host pointers are borrowed for the duration of a call only.
 *  - A context owns one CUDA stream and all of its device memory.  Calls on one
 *    context must not overlap; separate contexts are independent.
 *  - Nothing here allocates on the host side the caller must free.
 */
#ifndef LBFFS_CUDA_H
#define LBFFS_CUDA_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBFFS_OK 0
#define LBFFS_E_ARG (-1)     /* invalid argument (size, field id, enum value) */
#define LBFFS_E_CUDA (-2)    /* a CUDA runtime call failed; see lbffs_last_error */
#define LBFFS_E_STATE (-3)   /* call not valid in the current state */
#define LBFFS_E_UNSUPPORTED (-4) /* a combination the called entry point does not serve */
#define LBFFS_E_NONFINITE (-5)   /* a non-finite density was produced (divergence sentinel) */

typedef struct lbffs_ctx lbffs_ctx;

/* population storage in HBM; collision arithmetic is FP32 in every case */
enum lbffs_storage {
    LBFFS_FP32 = 0,  /* float, bit-compatible with the reference's buffers */
    LBFFS_FP16S = 1, /* IEEE half of (f_q - w_q) * 2^15 */
    LBFFS_BF16S = 2  /* bfloat16 of (f_q - w_q); below the 1e-3 velocity-error bar FP16S meets */
};
enum lbffs_collision {
    LBFFS_COLL_RR = 0,      /* recursive regularised (D3Q19 kernel.cl:3156; D3Q27: full Hermite basis) */
    LBFFS_COLL_CUMULANT = 1 /* Geier cumulant (D3Q27 kernel.cl:2352), D3Q27 only */
};
enum lbffs_sgs {
    LBFFS_SGS_SMAGORINSKY = 0, /* smagorinskyTauSGS with near-wall damping (kernel.cl:2133), honours LES */
    LBFFS_SGS_WALE = 1         /* waleTauSGS (kernel.cl:2267), the reference's live model; ignores LES */
};
enum lbffs_wall {
    LBFFS_WALL_BB = 0, /* half-way bounce-back on STL links (D3Q19 kernel.cl:1947) */
    LBFFS_WALL_IBB = 1 /* Filippova-Hanel / Mei-Luo-Shyy interpolated bounce-back (D3Q27 kernel.cl:1847-1888) */
};
/* near-wall damping of the Smagorinsky eddy viscosity (cells with a wall distance sdf, 0 < sdf != 10000) */
enum lbffs_damping {
    LBFFS_DAMP_WALL = 0,       /* min(1, kappa y / Cs)^2, kappa 0.41: the reference's live factor (kernel.cl:2170-2176) */
    LBFFS_DAMP_VAN_DRIEST = 1, /* min(1, (kappa / Cs) (1 - exp(-y+ / 26)) y)^2 with y+ from the log law (9.8 y+ = exp(kappa u+)):
                                  the block the reference keeps commented out (D3Q19 kernel.cl:2178-2197) */
    LBFFS_DAMP_NONE = 2        /* no damping */
};

/* Lattice description; replaces the compile-time choice of D3Q19_opencl vs D3Q27_opencl. */
typedef struct lbffs_desc {
    int nx, ny, nz;  /* input.txt nx ny nz */
    int q;           /* 19 or 27 */
    int storage;     /* enum lbffs_storage */
    int collision;   /* enum lbffs_collision */
    int sgs;         /* enum lbffs_sgs */
    int wall;        /* enum lbffs_wall */
    int device;      /* CUDA device ordinal */
    float cs;        /* Smagorinsky constant (the reference's live value is 0.1, kernel.cl:3628) */
    int damping;     /* enum lbffs_damping (0, the reference's factor, in a zero-initialised descriptor) */
} lbffs_desc;

/* Field ids: the reference's device buffers (ns.cpp:405-436). */
enum lbffs_field {
    LBFFS_F = 0,         /* float32[Q*E] populations (f_d); converted to/from the storage format.
                            An upload sets both population copies (f_d and fTmp_d), as initialization.hpp does. */
    LBFFS_BOUNDARY = 1,  /* int32[E] 1 on domain-face cells (boundary_d) */
    LBFFS_BOUNDARY1 = 2, /* int32[E] x-face BC code (boundary1_d), src/input.hpp:221-256 */
    LBFFS_BOUNDARY2 = 3, /* int32[E] y-face BC code */
    LBFFS_BOUNDARY3 = 4, /* int32[E] z-face BC code */
    LBFFS_SDF = 5,       /* float32[E] wall distance, 10000 = none (sdf_d) */
    LBFFS_SOLID = 6,     /* uint8[E] (solid_d) */
    LBFFS_NEISOLID = 7,  /* uint8[E] (neiSolid_d) */
    LBFFS_U0 = 8,        /* float32[E] wall / inlet velocity (u0_d) */
    LBFFS_V0 = 9,
    LBFFS_W0 = 10,
    LBFFS_OMEGA = 11,    /* float32[E] relaxation rate (omega_d) */
    LBFFS_TAUSGS = 12,   /* float32[E] eddy relaxation time (tauSGS_d) */
    LBFFS_RHO = 13,      /* float32[E] (rho_d) */
    LBFFS_U = 14,        /* float32[E] (u_d) */
    LBFFS_V = 15,
    LBFFS_W = 16,
    LBFFS_FWX = 17,      /* float32[E] STL-link wall force (Fwx_d) */
    LBFFS_FWY = 18,
    LBFFS_FWZ = 19,
    LBFFS_GXIBM = 20,    /* float32[E] IBM forcing field (GxIBM_d) */
    LBFFS_GYIBM = 21,
    LBFFS_GZIBM = 22,
    /* output step (lbffs_output): cal_rhoUVW of every cell at the last output, the host arrays
       rho / u / v / w of write.hpp:27 (download only; zeros before the first output) */
    LBFFS_OUT_RHO = 23,
    LBFFS_OUT_U = 24,
    LBFFS_OUT_V = 25,
    LBFFS_OUT_W = 26,
    /* time-mean accumulators uMean / vMean / wMean of write.hpp:70-76 (upload restores them) */
    LBFFS_UMEAN = 27,
    LBFFS_VMEAN = 28,
    LBFFS_WMEAN = 29,
    LBFFS_NFIELDS = 30
};

/* Per-step scalars: the trailing arguments of k_streamingCollision (ns.cpp:528-535). */
typedef struct lbffs_step_params {
    float dpdx;       /* lattice-unit pressure gradient (x) */
    float rho_av;     /* carried for interface parity; unused by the step, as in the reference */
    float les;        /* LES switch as float 0/1 */
    float omega_b;    /* bulk relaxation rate (omegaB, default 0.1) */
    float spz_width;  /* sponge width as a fraction of the domain (spzWidth, default 0.1) */
    float clim;       /* cumulant limiter (clim, default 0.01), D3Q27 */
    int store_fields; /* 0: macroscopic fields only where the step itself needs them;
                         1: rho/u/v/w/tauSGS of every fluid cell on the last step of the call;
                         2: on every step (what the reference does) */
} lbffs_step_params;

/* Create a context (replaces ns.cpp:385-436 context/queue/buffer creation).
   Device memory is zero-initialised except SDF = 10000 and OMEGA = 1. */
int lbffs_create(const lbffs_desc* desc, lbffs_ctx** out);
/* Release a context and all its device memory. */
int lbffs_destroy(lbffs_ctx* ctx);
/* Message of the last error on ctx (or on this thread if ctx is NULL). Never NULL. */
const char* lbffs_last_error(const lbffs_ctx* ctx);

/* Host -> device copy of one field (the cl::Buffer(context, begin, end, true) copies of
   ns.cpp:405-436).  bytes must equal the field size.  Geometry fields take effect at the
   next lbffs_step. */
int lbffs_upload(lbffs_ctx* ctx, int field, const void* host, size_t bytes);
/* Device -> host copy (cl::copy(queue, X_d, X.begin(), X.end()) of write.hpp:3-14). */
int lbffs_download(lbffs_ctx* ctx, int field, void* host, size_t bytes);

/* Advance nsteps time steps: each is one k_streamingCollision launch (ns.cpp:514-536), the
   IBM sub-step when markers are set (ns.cpp:542-601), and the f/fTmp swap (ns.cpp:602).
   Asynchronous on the context stream; errors of earlier launches are reported. */
int lbffs_step(lbffs_ctx* ctx, const lbffs_step_params* params, int nsteps);
/* Wait for the context stream (queue.finish()); reports the divergence sentinel. */
int lbffs_synchronize(lbffs_ctx* ctx);

/* FP64 sum of the STL-link wall force over fluid cells: SumFwx/y/z of write.hpp:25-46,
   accumulated in double instead of float. */
int lbffs_force_sum(lbffs_ctx* ctx, double out[3]);
/* FP64 sum of rho over fluid cells computed from the populations (write.hpp:25-46). */
int lbffs_mass(lbffs_ctx* ctx, double* out);

/* STL link table (bit q of mask set: population q of cell is a link, neiSolid && solid
   upwind, kernel.cl:1940-1943).  Writes min(n, capacity) entries in ascending cell order
   and the total count to *n.  Pass capacity 0 to query the count. */
int lbffs_links(lbffs_ctx* ctx, long long* cells, unsigned* masks, long long capacity, long long* n);

/* IBM markers (movingSTLcList, ns.cpp:248-254): n markers, xyz in lattice units. */
int lbffs_set_markers(lbffs_ctx* ctx, const float* xyz, int n);
int lbffs_get_markers(lbffs_ctx* ctx, float* xyz, int n);
/* Marker motion (readMotions, walls.hpp:586-629) plus an optional sinusoidal displacement
   amp*sin(2*pi*t/period) (period <= 0: none); t counts steps from set_motion. */
typedef struct lbffs_motion {
    float u_trans, v_trans, w_trans;    /* per-step translation */
    float rot_x, rot_y, rot_z;          /* rotation centre */
    float axis_x, axis_y, axis_z;       /* rotation axis (unit) */
    float rot_omega;                    /* rotation angle per step */
    float amp_x, amp_y, amp_z, period;  /* sinusoidal displacement */
} lbffs_motion;
int lbffs_set_motion(lbffs_ctx* ctx, const lbffs_motion* motion);
/* FP64 sum of the IBM forcing over fluid cells (SumGxIBM.. of write.hpp:25-46). */
int lbffs_ibm_force_sum(lbffs_ctx* ctx, double out[3]);

/* The context's cudaStream_t (for callers that order their own work after the step). */
int lbffs_get_stream(lbffs_ctx* ctx, void** stream);
/* Per-kernel device time (CUDA events around each launch) once enabled.  name is "bulk",
   "special" or "ibm"; returns accumulated milliseconds and launch count. */
int lbffs_set_timing(lbffs_ctx* ctx, int enabled);
int lbffs_kernel_time(lbffs_ctx* ctx, const char* name, double* total_ms, long long* launches);
/* Counts of cells per class after the geometry commit: [fluid, special, link, store]. */
int lbffs_cell_counts(lbffs_ctx* ctx, long long out[4]);

/* No counterpart in the reference (a choice between two implementations of the same D3Q19 step,
   which give identical results).  kind 0: each thread loads its cells' pulled populations from
   HBM; kind 1: a producer warp per CTA streams the pulled rows of each 256-cell row tile into a
   ring of shared-memory stages by bulk async copies and four consumer warps collide from there.
   D3Q27 contexts always use kind 0. */
int lbffs_set_bulk_kernel(lbffs_ctx* ctx, int kind);

/* No counterpart in the reference (a choice between two mappings of the same boundary kernel,
   which give identical results).  kind 0: one thread per cell of the special list; kind 1: a group
   of 16 lanes per cell, lane g doing the reads of directions g and g + 16; -1 (the default): kind 1 for lists of at most
   LBFFS_SPECIAL_WARP_MAX cells, where one thread per cell leaves most SMs idle, else kind 0.
   D3Q27 contexts always use kind 0. */
#define LBFFS_SPECIAL_WARP_MAX 16384
int lbffs_set_special_kernel(lbffs_ctx* ctx, int kind);

/* No counterpart in the reference (two ways to the same face streaming, which give identical
   results).  enabled 1 (the default): where every face carries one boundary code per axis (on a 2D
   grid: and the z faces carry no wall code, or both x faces are inlet / outlet / fixed-density /
   wall-function faces), the
   step kernels read each population that crosses the grid's border where the face streaming takes
   it (the periodic image, or the cell's own value of the bounce-back / mirror direction) instead of
   from a ghost layer filled before every step; where bulk cells lie on x faces without a Cyclic
   code, those cells write the x ghost slots they pull from next step themselves, and the ghost
   layer is filled once, before the first step after the populations were set from outside a step.
   0: the ghost-layer fill before every step, every cell pulling from a fixed offset. */
int lbffs_set_border_pulls(lbffs_ctx* ctx, int enabled);

/* setSolid + setNeiSolid (src/walls.hpp:159-216) on the device, bit for bit the reference's host
   result: solid[ic] = 1 for cells inside the closed surface (ray-crossing parity of isInner,
   walls.hpp:73-157, within the STL's bounding box, which the reference starts at the origin),
   inverted when invert != 0 (invertFluidSolid); neiSolid from solid as setNeiSolid builds it.
   vertices: ntri triangles x (v0, v1, v2) x (x, y, z) floats in lattice units, i.e. the STL's
   vertices after normalizeSTLv (stl.hpp:161-175), all patches concatenated.  Replaces the SOLID
   and NEISOLID fields; the geometry takes effect at the next lbffs_step. */
int lbffs_voxelize(lbffs_ctx* ctx, const float* vertices, long long ntri, int invert);

/* ---- Output step (D3Q19_opencl/write.hpp; D3Q27_opencl/write.hpp differs only in the restart
   file's population count) ---- */
typedef struct lbffs_output_params {
    float dpdx;        /* cal_rhoUVW's half-force shift (the step's dpdx) */
    float c;           /* velocity scale uMax / U0 of the VTK fields and of uAve */
    float L;           /* cell size of the VTK SPACING line and of the sdf / nuSGS fields */
    int out_interval;  /* outInterval: the weight of this output in the time means; 0 leaves them */
    int force_coeffs;  /* forceCoeffs: sum the wall and IBM forces, write the IBM fields (else zeros) */
} lbffs_output_params;

typedef struct lbffs_output_result {
    float rho_av;           /* rho_av_tmp / float(eleFluid) + 1 (write.hpp:47), the sum in FP64 */
    float rho_max, rho_min; /* over all cells (write.hpp:48-49) */
    float u_ave;            /* mean of u * c over the x = 0 plane, summed in the reference's float order */
    float time_mean;        /* timeMean after this output */
    long long n_fluid;      /* eleFluid */
    double fw[3];           /* SumFwx.. over fluid cells in FP64 (the reference sums in float) */
    double g_ibm[3];        /* SumGxIBM.. over fluid cells in FP64 */
} lbffs_output_result;

/* write.hpp:16-76 on the device: rho / u / v / w of every cell from the current populations by
   cal_rhoUVW (D3Q19.hpp:647-666, same float order) into LBFFS_OUT_*, the reductions above and, for
   out_interval > 0, uMean += u * outInterval.  Only the scalars leave the device. */
int lbffs_output(lbffs_ctx* ctx, const lbffs_output_params* params, lbffs_output_result* out);
/* The VTK file of write.hpp:78-600 from the last lbffs_output (ASCII, or binary with asciiToBinary's
   byte order, src/base.hpp:35-43).  Asynchronous: the call queues the device copies behind the work
   already on the context's stream and returns; a host thread writes the file while later steps
   run.  lbffs_io_wait (or the next output, upload, voxelisation, SDF or write call) joins it. */
int lbffs_write_vtk(lbffs_ctx* ctx, const char* path, int binary, const lbffs_output_params* params);
/* The restart file data.dat of write.hpp:603-631 (int nt, nx, ny, nz; then the populations q-major
   as float), from the current populations; asynchronous like lbffs_write_vtk (the populations are
   copied on the device first, so later steps do not change the file). */
int lbffs_write_restart(lbffs_ctx* ctx, const char* path, int nt);
/* restart.hpp: a data.dat of this grid into both population copies; *nt = its time step. */
int lbffs_read_restart(lbffs_ctx* ctx, const char* path, int* nt);
/* Wait for the asynchronous file write, if any; returns its error. */
int lbffs_io_wait(lbffs_ctx* ctx);

/* The LES wall-distance set-up of D3Q19_opencl/ns.cpp:200-225 on the device: the SDF field is set
   to sdf_ini, setSDF (src/walls.hpp:218-268, one call per STL patch) runs with (dr, p) around the
   context's current NEISOLID field, then setSDFnearBwalls (walls.hpp:372-467) with dr_walls on
   the uploaded BOUNDARY1..3 codes (int(dr_walls) < 0 skips it).  ns.cpp passes dr = 10, p = 7,
   sdf_ini = 10000, dr_walls = 3.  vertices: as for lbffs_voxelize, patches concatenated;
   normals: 3 floats per triangle, the facet normals as read from the STL; patch_ntri: npatch
   triangle counts.  Every setSDF call rewrites every near cell, so the result is that of the last
   patch's call (npatch = 0: no setSDF).  The arithmetic has the reference's types and order; the
   weight r^-p is computed in double on the device, so a sum may round differently from the host
   library's pow in rare cells (a float ulp).  Replaces the SDF field. */
int lbffs_build_sdf(lbffs_ctx* ctx, const float* vertices, const float* normals, const long long* patch_ntri,
                    int npatch, float dr, float p, float sdf_ini, float dr_walls);

/* Set both population copies to the rest equilibrium rho = 1, u = 0 (f_q = w_q), the state
   initialization.hpp writes for a fluid at rest, without a host upload of F. */
int lbffs_init_rest(lbffs_ctx* ctx);

/* ---- Serving: many solves resident on one GPU, advanced together ----
   The reference runs one case per process (ns.cpp); this server keeps many cases resident and
   advances all of them with one batched launch per kernel per step (CUDA graph replay), admitting
   queued cases as device memory and slots free up.  Each case is described exactly like a
   context (lbffs_desc + the reference's arrays) and computes the same numbers as lbffs_step.
   Supported: q = 19, RR collision, Smagorinsky SGS (LES on or off), BB or IBB walls, any storage;
   no IBM markers. */
typedef struct lbffs_server lbffs_server;

typedef struct lbffs_server_desc {
    int device;            /* CUDA device ordinal */
    size_t hbm_budget;     /* bytes of device memory the resident cases may hold */
    int max_cases;         /* resident cases at once */
    int steps_per_round;   /* steps per graph replay between admission / retirement checks */
} lbffs_server_desc;

/* One solve.  Array pointers are read during lbffs_server_submit only (copied).  boundary..
   boundary3 and solid / nei_solid are required; sdf, u0, v0, w0, omega may be NULL (10000, 0, 1);
   f NULL starts from rest (lbffs_init_rest). */
typedef struct lbffs_case {
    lbffs_desc desc;
    lbffs_step_params params;   /* store_fields is ignored: results hold the final step's fields */
    long long nsteps;
    int want_f;                 /* also keep the final populations */
    const int *boundary, *boundary1, *boundary2, *boundary3;
    const unsigned char *solid, *nei_solid;
    const float *sdf, *u0, *v0, *w0, *omega;
    const float* f;
} lbffs_case;

enum lbffs_case_state { LBFFS_CASE_QUEUED = 0, LBFFS_CASE_RUNNING = 1, LBFFS_CASE_DONE = 2, LBFFS_CASE_FAILED = -1 };

typedef struct lbffs_server_stats {
    long long submitted, completed, failed, resident, queued;
    long long rounds, graph_builds;
    double cell_updates;                        /* lattice updates of completed cases */
    double elapsed_s;                           /* first submission to last completion */
    double latency_p50_s, latency_p99_s, latency_mean_s, latency_max_s;  /* submit to result */
    double queue_wait_p50_s, queue_wait_p99_s;  /* submit to admission */
    size_t hbm_in_use, hbm_peak, hbm_capacity;
    double gpu_busy_s;        /* device time of the replayed rounds (CUDA events) */
    double build_s;           /* host time spent rebuilding batch tables and graphs */
    double mean_resident;     /* cases in the batch per round, averaged over rounds */
} lbffs_server_stats;

int lbffs_server_create(const lbffs_server_desc* desc, lbffs_server** out);
/* Stops the loop (cases still queued or running are abandoned) and frees everything. */
int lbffs_server_destroy(lbffs_server* srv);
/* Queue a solve; *id identifies it in the calls below.  LBFFS_E_UNSUPPORTED for a case outside the
   supported set, LBFFS_E_ARG when it can never fit the budget. */
int lbffs_server_submit(lbffs_server* srv, const lbffs_case* c, long long* id);
/* Current state (enum lbffs_case_state). */
int lbffs_server_poll(lbffs_server* srv, long long id, int* state);
/* Block until the case is done or failed, or timeout_s passes (LBFFS_E_STATE on timeout). */
int lbffs_server_wait(lbffs_server* srv, long long id, double timeout_s);
/* Copy a result field of a finished case: LBFFS_RHO, LBFFS_U, LBFFS_V, LBFFS_W (float32[E]) or
   LBFFS_F (float32[Q*E], when want_f was set). */
int lbffs_server_result(lbffs_server* srv, long long id, int field, void* host, size_t bytes);
/* Drop a finished case's results. */
int lbffs_server_release(lbffs_server* srv, long long id);
int lbffs_server_get_stats(lbffs_server* srv, lbffs_server_stats* out);
/* Message of the last failure of case id (or of the server when id < 0). */
const char* lbffs_server_error(lbffs_server* srv, long long id);

/* No counterpart in the reference.  FP64 sum of rho over fluid cells (solid[ic] == 0) of float32
   populations f[q*n_cells + ic] that the caller holds on `device`, written to the caller's
   device double `out` in stream order on `stream` (0: the legacy default stream).  It is the
   lbffs_mass reduction for callers that cannot allocate device memory when they need the check
   (a serving loop holding a fixed HBM budget, a driver that owns its own buffers and has no
   context): it calls no allocating routine and uses a fixed 256 KiB scratch array that every GPU
   loading this library keeps until exit.  The first call on a device looks up that array (and may
   load the library's device code there); make it before any stream capture.  That address is kept
   per device for the life of the process, so the device's primary context must not be reset
   (cudaDeviceReset) between calls.  n_cells above LBFFS_NOALLOC_MAX_CELLS, q other than 19 or 27,
   null pointers and device ordinals of 64 or more are rejected with LBFFS_E_ARG before anything is
   launched.  The caller's current device is the same after the call as before it.  Calls share
   the scratch: calls whose kernels overlap on the GPU race.  Errors are reported by
   lbffs_last_error(NULL). */
#define LBFFS_NOALLOC_MAX_CELLS 268435456
int lbffs_mass_noalloc(int device, const float* f, const unsigned char* solid, int q, long long n_cells,
                       double* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif
