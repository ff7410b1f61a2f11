/*
 * fv2d_gpu.h -- C ABI of the GB300 (sm_103a) finite-volume residual-and-update library.
 *
 * Drop-in for the solver step of Avery-Hantla/CFD-2D-NS-FV (fv2d).  The reference selects its
 * solver at link time (CMakeLists.txt:17-25,92-96) and calls free C++ functions on host objects;
 * this library keeps the mesh and the state resident on one GPU and exposes plain-C entry
 * points: pointers, sizes and int status codes, no C++ or torch types, no exceptions, no exit().
 * A handle owns one CUDA stream and one device allocation; handles are independent.
 *
 * Conventions
 *   - cell arrays exchanged with the host use the reference's own (file) numbering and its SoA
 *     layout: p1[0..N), p2[0..N), p3[0..N), p4[0..N) (class_Q, src/support/class_q.hpp:15-18);
 *   - mesh input uses the grid_file.in conventions (src/base/readmesh.cpp:31-85): 1-based point
 *     and cell ids, face_cell2 = 0 for BC1 faces and -1 for BC2 faces;
 *   - every function returns FV2D_OK (0) or a positive error code; fv2d_last_error() gives text.
 */
#ifndef FV2D_GPU_H
#define FV2D_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define FV2D_OK             0
#define FV2D_ERR_ARG        1   /* invalid argument or handle                                   */
#define FV2D_ERR_IO         2   /* input.in / grid file could not be opened or parsed           */
#define FV2D_ERR_MESH       3   /* mesh rejected (ids out of range, unsupported ordering)       */
#define FV2D_ERR_CASE       4   /* option the solver step does not implement (order 3, ...)     */
#define FV2D_ERR_CUDA       5   /* CUDA runtime error                                           */
#define FV2D_ERR_NOMEM      6   /* device memory exhausted                                      */
#define FV2D_ERR_STATE      7   /* non-physical state detected (NaN, rho <= 0 or P <= 0)        */
#define FV2D_ERR_NODEV      8   /* no CUDA device / the library's kernels cannot run here       */

#define FV2D_FP64 0             /* plain FP64 path, bit-exact with the reference                */
#define FV2D_FP32 1             /* FP32 state/gradients/fluxes; LSQ terms from FP64; FP64 norms */

/* Codes as read_inputs maps them (src/base/read_inputs.cpp:44-206). */
#define FV2D_EULER 1
#define FV2D_NS 2
#define FV2D_RUSANOV 1
/* ROE is run as the reference runs it: its res() calls no flux routine (res.cpp:62-69), so every
 * face's inviscid flux is class_F::init's -101 (class_f.hpp:26-30) and the time step keeps the
 * initial spectral terms (class_q.hpp:61-62); only the NS viscous flux is computed.             */
#define FV2D_ROE 2
#define FV2D_LIM_NONE 0
#define FV2D_LIM_MINMOD 1
#define FV2D_LIM_SQUEEZE 2
#define FV2D_DT_GLOBAL 1
#define FV2D_DT_LOCAL 2
#define FV2D_SSP_RK2 1
#define FV2D_SSP_RK3 2
#define FV2D_BC_FREESTREAM (-1)
#define FV2D_BC_SLIP_WALL (-2)
#define FV2D_BC_EXTRAPOLATION (-3)
#define FV2D_BC_NO_SLIP_WALL (-4)

/* The contents of input.in after read_inputs (struct_inputs, struct_time, struct_BC,
 * struct_report and the class_flow fields it sets: src/support/struct_*.hpp, class_flow.hpp). */
typedef struct fv2d_case {
    int order;                  /* solution_poly_order + 1 (read_inputs.cpp:26)          */
    int nmax, monitor_step, output_step, restart;
    int eqn, flux_solver, limiter;
    int time_type, time_scheme;
    int bc1, bc2;
    double cfl;
    double gamma, R, mu, Pr;    /* [fluid]  */
    double P, rho, u, v;        /* [init]   */
    double length;              /* [report] */
    char grid_file[4096];
} fv2d_case;

/* A mesh in grid_file.in conventions (arrays are read during the call only). */
typedef struct fv2d_mesh_desc {
    int num_points, num_faces, num_cells;
    const double* x;
    const double* y;
    const int* face_point1;
    const int* face_point2;
    const int* face_cell1;
    const int* face_cell2;
} fv2d_mesh_desc;

typedef struct fv2d_handle fv2d_handle;
typedef struct fv2d_mesh fv2d_mesh;

/* ---- input surface (host only; no GPU needed) ---------------------------------------------- */

/* Parse input.in.  Replaces read_inputs() (src/base/read_inputs.cpp:10).                        */
int fv2d_read_inputs(const char* path, fv2d_case* out);

/* Parse grid_file.in into caller-visible arrays.  Replaces the parse half of readmesh()
 * (src/base/readmesh.cpp:18-111).  *out_* are allocated with malloc; free with fv2d_free(). */
int fv2d_read_grid(const char* path, int* num_points, int* num_faces, int* num_cells,
                   double** x, double** y, int** face_point1, int** face_point2,
                   int** face_cell1, int** face_cell2);
void fv2d_free(void* p);
/* Write a mesh in the grid_file.in format readmesh() reads (src/base/readmesh.cpp:31-70); point
 * coordinates with 17 significant digits, so fv2d_read_grid returns the same doubles.  Host only. */
int fv2d_write_grid(const char* path, const fv2d_mesh_desc* desc);

/* Host mesh build: connectivity, BC tagging and geometry exactly as readmesh()
 * (src/base/readmesh.cpp:31-411), plus the cell/face renumbering used on the device.          */
int fv2d_mesh_build(const fv2d_mesh_desc* desc, const fv2d_case* cs, fv2d_mesh** out);
void fv2d_mesh_free(fv2d_mesh* m);
/* sizes: num_points, num_faces, num_cells, numBC1, numBC2, numWALL, num_of_BC, max_sides      */
int fv2d_mesh_sizes(const fv2d_mesh* m, int* out8);
/* geometry in the reference's numbering; field ids as in fv2d_field (FV2D_G_*)               */
int fv2d_mesh_get(const fv2d_mesh* m, int field, double* out);
/* permutations: kind 0 = cell new->old (N), 1 = face new->old (F)                             */
int fv2d_mesh_permutation(const fv2d_mesh* m, int kind, int* out);
/* The FP32 engine's tile layout of a mesh (host only; no counterpart in the reference, whose
 * solver has no device layout): builds it, checks that every index its stage kernels derive stays
 * in range (FV2D_ERR_MESH otherwise) and reports tiles, record words, records, csr words, halo ids,
 * face records with fluxes, ring-1 cells and ring-2 cells (out8).                               */
int fv2d_mesh_tiles(const fv2d_mesh* m, long long* out8);

/* ---- solver (GPU) ------------------------------------------------------------------------- */

/* Create a solver: upload mesh + uniform freestream state (main.cpp:75-118).  precision is
 * FV2D_FP64 or FV2D_FP32.  Replaces the setup half of main() and the arguments the reference
 * threads through ssp_rk3() (src/include/ssp_rk3.hpp:1).                                       */
int fv2d_create(const fv2d_mesh_desc* desc, const fv2d_case* cs, int precision, fv2d_handle** out);
/* Same, from an input.in path (read_inputs + readmesh).                                        */
int fv2d_create_from_files(const char* input_path, int precision, fv2d_handle** out);
void fv2d_destroy(fv2d_handle* h);

/* Advance `iterations` SSP-RK3 iterations.  Replaces ssp_rk3() (src/solver/ssp_rk3.cpp:18),
 * which main() calls once per iteration (src/base/main.cpp:121-133).  Asynchronous on the
 * handle's stream; errors from device-side checks surface at the next synchronizing call.     */
int fv2d_step(fv2d_handle* h, int iterations);
/* Advance one RK stage (one res() call, src/solver/res.cpp:21, plus its stage combination).   */
int fv2d_stage(fv2d_handle* h);

/* Restart path (main.cpp:82-106): replace Qbar by q (4N, SoA, file numbering) and recompute the
 * primitives; face histories are reset as for a fresh run.                                    */
int fv2d_set_state(fv2d_handle* h, const double* q);
/* Replace Qbar by q (4N, SoA, file numbering) WITHOUT resetting the face histories the next
 * stage reads (previous-stage face values, Vn_avg/c_avg).  For a host loop that hands back the
 * state it read with fv2d_get_state, as the reference's main() hands Qbar to ssp_rk3() every
 * iteration (src/base/main.cpp:126): upload, step, download continues the run exactly.        */
int fv2d_load_state(fv2d_handle* h, const double* q);
/* Copy Qbar back (4N, SoA, file numbering).                                                    */
int fv2d_get_state(fv2d_handle* h, double* q);
/* Read a field (fv2d_field ids); blocks until the stream is idle.                              */
int fv2d_get_field(fv2d_handle* h, int field, double* out);
/* L2 norms of the residual of the last stage (src/base/save_sol.cpp:79-89).                   */
int fv2d_residual_norm(fv2d_handle* h, double out4[4]);
/* sizes: num_points, num_faces, num_cells, numBC1, numBC2, numWALL, num_of_BC, stage          */
int fv2d_sizes(fv2d_handle* h, int* out8);

/* ---- solution files (the reference's layout, written in the working directory's sol/ and mesh/) */
/* Monitor line (stdout) + sol/output.dat + sol/res_history.dat every monitor_step, and the
 * node-averaged Tecplot volume/surface files every output_step, for iteration `ndx`.  Replaces
 * save() (src/base/save_sol.cpp:16); call it after the iteration's fv2d_step.                  */
int fv2d_save(fv2d_handle* h, int ndx);
/* sol/restart_sol.dat for iteration `ndx`.  Replaces post() (src/base/post_process.cpp:13).   */
int fv2d_post(fv2d_handle* h, int ndx);
/* Headers of sol/res_history.dat and sol/output.dat (src/base/main.cpp:59-73).                */
int fv2d_write_history_headers(fv2d_handle* h);
/* mesh/cell_data.dat and mesh/face_data.dat (src/base/readmesh.cpp:413-446).                  */
int fv2d_write_mesh_files(fv2d_handle* h);
/* Checkpoint: the current Qbar in the restart_sol.dat layout (post_process.cpp:17-27) to `path`
 * with `digits` significant digits (0: the reference's 6; 17: every double round-trips exactly
 * through fv2d_read_restart + fv2d_set_state).                                                 */
int fv2d_write_restart(fv2d_handle* h, const char* path, int ndx, int digits);
/* Read sol/restart_sol.dat-format file into q (4N SoA); *ndx = the iteration it was written at
 * (src/base/main.cpp:82-104).  Host only.                                                      */
int fv2d_read_restart(const char* path, int num_cells, int* ndx, double* q);
int fv2d_synchronize(fv2d_handle* h);
/* Store the residual after every stage (parity checks) instead of only after the last stage.  */
int fv2d_set_store_residual(fv2d_handle* h, int every_stage);
/* Capture full iterations in a CUDA graph (default on).                                        */
int fv2d_set_graphs(fv2d_handle* h, int enable);
/* Time every kernel launch with CUDA events on the handle's stream (off by default).          */
int fv2d_set_kernel_timing(fv2d_handle* h, int enable);
/* Per-kernel totals since timing was enabled: names (comma separated into buf), ms, launches. */
int fv2d_kernel_times(fv2d_handle* h, char* names, int names_len, double* ms, int* launches, int max_kernels, int* n_kernels);
/* The handle's CUDA stream (a cudaStream_t), for callers that order their own work after it.  */
void* fv2d_stream(fv2d_handle* h);
/* Device bytes held by the handle.                                                             */
long long fv2d_device_bytes(fv2d_handle* h);

const char* fv2d_last_error(fv2d_handle* h);   /* h may be NULL: last creation error */

/* ---- batched solves (many independent solves resident on one GPU) ----------------------------
 * No single counterpart in the reference, which runs one solve per process; each solve in a batch
 * advances exactly as ssp_rk3() (src/solver/ssp_rk3.cpp:18) would advance it alone.  A batch owns
 * one device arena sized at creation (cells, faces, solves); solves are added (mesh + case, the
 * same inputs as fv2d_create) and removed between iterations; fv2d_batch_step advances every
 * active solve together with one persistent launch per kernel per RK stage, replayed as one CUDA
 * graph per iteration.  Per-solve residual L2 norms of the last iteration support retirement.
 * Errors: fv2d_last_error(NULL).                                                                 */
typedef struct fv2d_batch fv2d_batch;
int fv2d_batch_create(long long max_cells, long long max_faces, int max_solves, int precision, fv2d_batch** out);
void fv2d_batch_destroy(fv2d_batch* b);
/* device bytes a solve with this mesh occupies in a batch of the given precision (admission)   */
int fv2d_batch_footprint(const fv2d_mesh_desc* desc, int precision, long long* bytes);
/* FV2D_ERR_NOMEM when the arena has no room (the batch is unchanged)                           */
int fv2d_batch_add(fv2d_batch* b, const fv2d_mesh_desc* desc, const fv2d_case* cs, int* solve_id);
/* the same from a host mesh built by fv2d_mesh_build with the same BC codes (lets a caller build
 * meshes ahead of admission, or reuse one for solves that differ only in flow conditions)      */
int fv2d_batch_add_mesh(fv2d_batch* b, const fv2d_mesh* mesh, const fv2d_case* cs, int* solve_id);
int fv2d_batch_remove(fv2d_batch* b, int solve_id);
int fv2d_batch_step(fv2d_batch* b, int iterations);
/* for every active solve: id, the 4 residual L2 norms of its last iteration (summed in a fixed
 * order, so reproducible bit for bit; meaningful once iterations > 0), iterations done         */
int fv2d_batch_norms(fv2d_batch* b, int* solve_ids, double* norms4, int* iterations, int max, int* n);
int fv2d_batch_get_state(fv2d_batch* b, int solve_id, double* q);
int fv2d_batch_synchronize(fv2d_batch* b);
/* launch shape per solve-size bucket (buckets split at bucket_edges[0] and bucket_edges[1] cells);
 * results never depend on it.  FP64: threads per block (a multiple of 32 in [64, 256]) and tiles
 * of block * tile_mult[bucket] elements.  FP32 (fused stage kernel over the mesh's 256-cell tiles,
 * 256 threads per tile): block is not used; tile_mult[bucket] in [1, 32] sets the faces per warp of
 * the flux pass (32 * tile_mult flux records per grab).                                          */
int fv2d_batch_set_tuning(fv2d_batch* b, int block, const int* tile_mult3, const int* bucket_edges2);
int fv2d_batch_get_tuning(fv2d_batch* b, int* block, int* tile_mult3, int* bucket_edges2);
/* grid of the stage kernels: 0 = persistent (SMs x resident blocks loop over the tiles),
 * 1 = one block per tile (the graph is re-captured when the tile count changes)                 */
int fv2d_batch_set_grid_mode(fv2d_batch* b, int full_grid);
/* cells used/capacity, faces used/capacity, incidences used/capacity, active solves, bytes      */
int fv2d_batch_usage(fv2d_batch* b, long long* out8);
int fv2d_batch_set_kernel_timing(fv2d_batch* b, int enable);
/* totals since timing was enabled for gradient, face and update kernels                        */
int fv2d_batch_kernel_times(fv2d_batch* b, double* ms3, int* launches3);
void* fv2d_batch_stream(fv2d_batch* b);

/* ---- residual without allocation ----------------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device memory: a host
 * application whose own allocator has reserved the GPU's memory up front (a cudaMalloc here would
 * fail or fragment its pool), or a latency-critical thread that must not call cudaMalloc/cudaFree
 * because they can synchronise the whole device.  The caller passes every input and output as
 * device memory it already owns; the call computes the FIRST-ORDER residual (res() with
 * solution_poly_order = 0, src/solver/res.cpp:21: boundary ghosts, Rusanov flux, gather / volume;
 * no viscous flux, as in the reference at first order) and allocates nothing.
 *
 * Its per-face scratch is a static device array of FV2D_NOALLOC_MAX_FACES x 4 doubles (8 MiB)
 * that lives with the library's device code on each GPU until the process exits; meshes with more
 * faces are rejected with FV2D_ERR_ARG (use fv2d_create / fv2d_stage for those).  The first call on
 * each device looks up that array's device address with the device current; make that first call
 * before any stream capture.  Under CUDA's lazy module loading (the default; CUDA_MODULE_LOADING
 * unset or LAZY) the library's device code and this array are only placed on a device by that first
 * call, so the FIRST call does take device memory: a host whose allocator reserves the GPU's memory
 * makes one warm-up call per device (any small mesh) before it reserves its pool, or runs with
 * CUDA_MODULE_LOADING=EAGER.  Every later call allocates nothing.  The looked-up address belongs to
 * the device's primary context: resetting the device (cudaDeviceReset) after the first call is not
 * supported in the same process.  The scratch is fully rewritten before it is read, so no state
 * carries over between calls, but all calls share it: calls that overlap on the GPU (other
 * streams, other host threads on the same device) race and must be serialised by the caller.
 * The kernels are launched on `stream` (a cudaStream_t, NULL = legacy default stream) and the call
 * returns without waiting; errors: fv2d_last_error(NULL).
 *
 * Mesh arrays use the reference's numbering and codes, 0-based, and must be in range (they are
 * not checked on the device): face_cell1 in [0, num_cells); face_cell2 in [0, num_cells) for an
 * interior face or one of the BC codes -1 (FREESTREAM), -2 (SLIP_WALL), -3 (EXTRAPOLATION),
 * -4 (NO_SLIP_WALL); cell_face_offsets non-decreasing from 0; cell_faces holds
 * (face id << 1) | side (side 1 when the cell is face_cell2) with face ids in [0, num_faces), in
 * ascending face id per cell, which reproduces the reference's summation order; q and r are SoA
 * p1..p4 blocks of num_cells doubles.  From the case only gamma, the [init] state and
 * flux_solver are read (RUSANOV only: ROE is rejected with FV2D_ERR_CASE). */
#define FV2D_NOALLOC_MAX_FACES 262144
typedef struct fv2d_noalloc_mesh {
    int num_cells, num_faces;
    const int* face_cell1;          /* device [num_faces]                       */
    const int* face_cell2;          /* device [num_faces]                       */
    const double* face_nx;          /* device [num_faces]                       */
    const double* face_ny;          /* device [num_faces]                       */
    const double* face_area;        /* device [num_faces]                       */
    const int* cell_face_offsets;   /* device [num_cells + 1]                   */
    const int* cell_faces;          /* device [cell_face_offsets[num_cells]]    */
    const double* cell_vol;         /* device [num_cells]                       */
} fv2d_noalloc_mesh;
int fv2d_residual_noalloc(const fv2d_noalloc_mesh* mesh, const fv2d_case* cs, const double* q, double* r,
                          void* stream);

/* Field ids for fv2d_get_field / fv2d_mesh_get (same numbering as the oracle's interface).     */
enum fv2d_field {
    FV2D_F_QBAR = 0,        /* 4N  Qbar                                                  */
    FV2D_F_QSTAR = 1,       /* 4N  Q* (output of stage 1, then of stage 2)               */
    FV2D_F_RES = 2,         /* 4N  residual of the last stage                            */
    FV2D_F_DT = 3,          /* N   time step of the current iteration                    */
    FV2D_F_QBAR_GRAD = 4,   /* 8N  limited gradient of Qbar (stage 1 of this iteration)  */
    FV2D_F_QSTAR_GRAD = 5,  /* 8N  limited gradient of Q* (last stage 2 or 3 input)      */
    FV2D_G_AREA = 20, FV2D_G_NX, FV2D_G_NY, FV2D_G_FCX, FV2D_G_FCY,
    FV2D_G_C1DX, FV2D_G_C1DY, FV2D_G_C2DX, FV2D_G_C2DY, FV2D_G_DXJ, FV2D_G_DYJ,
    FV2D_G_DIST, FV2D_G_LX, FV2D_G_LY, FV2D_G_MX, FV2D_G_MY,
    FV2D_G_VOL = 40, FV2D_G_CCX, FV2D_G_CCY, FV2D_G_IXX, FV2D_G_IYY, FV2D_G_IXY, FV2D_G_DELTA,
    FV2D_G_BCCX = 50, FV2D_G_BCCY
};

#ifdef __cplusplus
}
#endif
#endif
