// C ABI of the GB300 fv2d library (declared in include/fv2d_gpu.h).
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>
#include <string>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>   // header-only; ranges are free unless a profiler attaches

#include "fv2d_gpu.h"
#include "fv2d_host.h"
#include "fv2d_output.h"
#include "fv2d_batch.h"
#include "fv2d_solver.h"
#include "fv2d_tiles.h"

namespace {
// Named NVTX range around a C-ABI call (shows the library's calls on an Nsight timeline).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};
}  // namespace

namespace fv2d {
const char* const kKernelNames[K_COUNT] = {"k_gradient", "k_face", "k_update", "k_spectral_init",
                                          "k_state_in", "k_state_out", "k_res_norm_partial", "k_tstage"};
}

struct fv2d_handle {
    std::unique_ptr<fv2d::Solver> s;
    int precision = FV2D_FP64;
    fv2d_case cs{};
};

struct fv2d_mesh {
    fv2d::HostMesh m;
};

struct fv2d_batch {
    std::unique_ptr<fv2d::Batch> b;
    int precision = FV2D_FP32;
};

namespace {
thread_local std::string g_err;
}  // namespace

namespace fv2d {
void set_global_error(const std::string& msg) { g_err = msg; }
}  // namespace fv2d

namespace {

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

// Options the reference's solver step implements (res.cpp:26-69, ssp_rk3.cpp, main.cpp:122-127).
int check_case(const fv2d_case* cs) {
    if (!cs) return fail(FV2D_ERR_ARG, "null case");
    if (cs->order != 1 && cs->order != 2)
        return fail(FV2D_ERR_CASE, "solution_poly_order must be 0 or 1 (res.cpp:56-58 rejects other orders)");
    if (cs->eqn != FV2D_EULER && cs->eqn != FV2D_NS) return fail(FV2D_ERR_CASE, "eqn must be EULER or NS");
    if (cs->flux_solver != FV2D_RUSANOV && cs->flux_solver != FV2D_ROE)
        return fail(FV2D_ERR_CASE, "flux_solver must be RUSANOV or ROE");
    if (cs->limiter != FV2D_LIM_NONE && cs->limiter != FV2D_LIM_MINMOD && cs->limiter != FV2D_LIM_SQUEEZE)
        return fail(FV2D_ERR_CASE, "limiter must be NONE, MINMOD or SQUEEZE");
    if (cs->time_type != FV2D_DT_GLOBAL && cs->time_type != FV2D_DT_LOCAL)
        return fail(FV2D_ERR_CASE, "time_step_type must be GLOBAL or LOCAL");
    for (int b : {cs->bc1, cs->bc2})
        if (b > -1 || b < -4) return fail(FV2D_ERR_CASE, "BC1/BC2 must be FREESTREAM, SLIP_WALL, EXTRAPOLATION or NO_SLIP_WALL");
    if (!(cs->gamma > 1) || !(cs->R > 0) || !(cs->rho > 0) || !(cs->P > 0))
        return fail(FV2D_ERR_CASE, "gamma > 1, R > 0, rho > 0 and P > 0 are required");
    if (cs->eqn == FV2D_NS && !(cs->Pr > 0)) return fail(FV2D_ERR_CASE, "NS needs Pr > 0");
    if (!(cs->cfl > 0)) return fail(FV2D_ERR_CASE, "CFL must be > 0");
    return FV2D_OK;
}

int check_device() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return fail(FV2D_ERR_NODEV, std::string("no CUDA device: ") + cudaGetErrorString(e));
    return FV2D_OK;
}
}  // namespace

extern "C" {

int fv2d_read_inputs(const char* path, fv2d_case* out) {
    if (!path || !out) return fail(FV2D_ERR_ARG, "null argument");
    std::string err;
    int rc = fv2d::parse_inputs(path, out, err);
    if (rc) g_err = err;
    return rc;
}

int fv2d_read_grid(const char* path, int* num_points, int* num_faces, int* num_cells, double** x, double** y,
                   int** face_point1, int** face_point2, int** face_cell1, int** face_cell2) {
    if (!path || !num_points || !num_faces || !num_cells || !x || !y || !face_point1 || !face_point2 || !face_cell1 || !face_cell2)
        return fail(FV2D_ERR_ARG, "null argument");
    std::vector<double> vx, vy;
    std::vector<int> a, b, c, d;
    int nc = 0;
    std::string err;
    int rc = fv2d::parse_grid(path, vx, vy, a, b, c, d, nc, err);
    if (rc) return fail(rc, err);
    auto dup = [](const void* src, size_t bytes) { void* p = std::malloc(bytes ? bytes : 1); std::memcpy(p, src, bytes); return p; };
    *num_points = (int)vx.size(); *num_faces = (int)a.size(); *num_cells = nc;
    *x = (double*)dup(vx.data(), 8 * vx.size());
    *y = (double*)dup(vy.data(), 8 * vy.size());
    *face_point1 = (int*)dup(a.data(), 4 * a.size());
    *face_point2 = (int*)dup(b.data(), 4 * b.size());
    *face_cell1 = (int*)dup(c.data(), 4 * c.size());
    *face_cell2 = (int*)dup(d.data(), 4 * d.size());
    return FV2D_OK;
}

void fv2d_free(void* p) { std::free(p); }

int fv2d_write_grid(const char* path, const fv2d_mesh_desc* d) {
    if (!path || !d || !d->x || !d->y || !d->face_point1 || !d->face_point2 || !d->face_cell1 || !d->face_cell2)
        return fail(FV2D_ERR_ARG, "null argument");
    std::string err;
    const int rc = fv2d::write_grid(path, d, err);
    return rc ? fail(rc, err) : FV2D_OK;
}

int fv2d_mesh_build(const fv2d_mesh_desc* desc, const fv2d_case* cs, fv2d_mesh** out) {
    if (!out) return fail(FV2D_ERR_ARG, "null output");
    *out = nullptr;
    int rc = check_case(cs);
    if (rc) return rc;
    auto m = std::make_unique<fv2d_mesh>();
    std::string err;
    rc = fv2d::build_mesh(desc, cs, m->m, err);
    if (rc) return fail(rc, err);
    *out = m.release();
    return FV2D_OK;
}

void fv2d_mesh_free(fv2d_mesh* m) { delete m; }

int fv2d_mesh_sizes(const fv2d_mesh* mm, int* o) {
    if (!mm || !o) return fail(FV2D_ERR_ARG, "null argument");
    const fv2d::HostMesh& m = mm->m;
    o[0] = m.np; o[1] = m.nf; o[2] = m.nc; o[3] = m.numBC1; o[4] = m.numBC2; o[5] = m.numWALL;
    o[6] = m.num_of_BC; o[7] = m.max_sides;
    return FV2D_OK;
}

int fv2d_mesh_get(const fv2d_mesh* mm, int field, double* out) {
    if (!mm || !out) return fail(FV2D_ERR_ARG, "null argument");
    return fv2d::mesh_field(mm->m, field, out) < 0 ? fail(FV2D_ERR_ARG, "unknown mesh field") : FV2D_OK;
}

int fv2d_mesh_permutation(const fv2d_mesh* mm, int kind, int* out) {
    if (!mm || !out) return fail(FV2D_ERR_ARG, "null argument");
    const std::vector<int>& p = kind == 0 ? mm->m.cell_new2old : mm->m.face_new2old;
    std::copy(p.begin(), p.end(), out);
    return FV2D_OK;
}

int fv2d_mesh_tiles(const fv2d_mesh* mm, long long* o) {
    if (!mm || !o) return fail(FV2D_ERR_ARG, "null argument");
    fv2d::DeviceLayout L;
    fv2d::build_layout(mm->m, L);
    fv2d::TileLayout T;
    std::string err;
    if (!fv2d::build_tile_layout(mm->m, L, T, err)) return fail(FV2D_ERR_MESH, err);
    long long nrc = 0, r1 = 0, r2 = 0;
    for (const auto& t : T.tiles) { nrc += t.nrc; r1 += t.n1; r2 += t.n2; }
    o[0] = (long long)T.tiles.size(); o[1] = (long long)T.rec.size(); o[2] = (long long)T.qcell.size();
    o[3] = (long long)T.csr.size(); o[4] = (long long)T.halo.size(); o[5] = nrc; o[6] = r1; o[7] = r2;
    return FV2D_OK;
}

int fv2d_create(const fv2d_mesh_desc* desc, const fv2d_case* cs, int precision, fv2d_handle** out) {
    NvtxRange nvtx_("fv2d_create");
    if (!out) return fail(FV2D_ERR_ARG, "null output");
    *out = nullptr;
    int rc = check_case(cs);
    if (rc) return rc;
    if (precision != FV2D_FP64 && precision != FV2D_FP32) return fail(FV2D_ERR_ARG, "precision must be FV2D_FP64 or FV2D_FP32");
    if ((rc = check_device())) return rc;
    auto h = std::make_unique<fv2d_handle>();
    h->precision = precision;
    h->s.reset(precision == FV2D_FP64 ? fv2d::make_solver_fp64() : fv2d::make_solver_fp32());
    std::string err;
    rc = fv2d::build_mesh(desc, cs, h->s->mesh_, err);
    if (rc) return fail(rc, err);
    rc = h->s->init(*cs);
    if (rc) return fail(rc, h->s->err_);
    h->cs = *cs;
    *out = h.release();
    return FV2D_OK;
}

int fv2d_create_from_files(const char* input_path, int precision, fv2d_handle** out) {
    if (!input_path || !out) return fail(FV2D_ERR_ARG, "null argument");
    *out = nullptr;
    fv2d_case cs;
    int rc = fv2d_read_inputs(input_path, &cs);
    if (rc) return rc;
    std::vector<double> x, y;
    std::vector<int> a, b, c, d;
    int nc = 0;
    std::string err;
    rc = fv2d::parse_grid(cs.grid_file, x, y, a, b, c, d, nc, err);   // relative to the working directory, like readmesh
    if (rc) return fail(rc, err);
    fv2d_mesh_desc desc{(int)x.size(), (int)a.size(), nc, x.data(), y.data(), a.data(), b.data(), c.data(), d.data()};
    return fv2d_create(&desc, &cs, precision, out);
}

void fv2d_destroy(fv2d_handle* h) { delete h; }

#define FV2D_H(h) if (!(h) || !(h)->s) return fail(FV2D_ERR_ARG, "null handle")
#define FV2D_RET(h, expr) do { int rc_ = (expr); if (rc_) g_err = (h)->s->err_; return rc_; } while (0)

int fv2d_step(fv2d_handle* h, int iterations) { NvtxRange r("fv2d_step"); FV2D_H(h); FV2D_RET(h, h->s->step(iterations)); }
int fv2d_stage(fv2d_handle* h) { NvtxRange r("fv2d_stage"); FV2D_H(h); FV2D_RET(h, h->s->stage()); }

int fv2d_set_state(fv2d_handle* h, const double* q) {
    NvtxRange nvtx_("fv2d_set_state");
    FV2D_H(h);
    if (!q) return fail(FV2D_ERR_ARG, "null state");
    FV2D_RET(h, h->s->set_state(q));
}

int fv2d_load_state(fv2d_handle* h, const double* q) {
    NvtxRange nvtx_("fv2d_load_state");
    FV2D_H(h);
    if (!q) return fail(FV2D_ERR_ARG, "null state");
    FV2D_RET(h, h->s->load_state(q));
}

int fv2d_get_state(fv2d_handle* h, double* q) {
    NvtxRange nvtx_("fv2d_get_state");
    FV2D_H(h);
    if (!q) return fail(FV2D_ERR_ARG, "null output");
    FV2D_RET(h, h->s->get_field(FV2D_F_QBAR, q));
}

int fv2d_get_field(fv2d_handle* h, int field, double* out) {
    FV2D_H(h);
    if (!out) return fail(FV2D_ERR_ARG, "null output");
    FV2D_RET(h, h->s->get_field(field, out));
}

int fv2d_residual_norm(fv2d_handle* h, double out4[4]) {
    FV2D_H(h);
    if (!out4) return fail(FV2D_ERR_ARG, "null output");
    FV2D_RET(h, h->s->residual_norm(out4));
}

int fv2d_sizes(fv2d_handle* h, int* o) {
    FV2D_H(h);
    if (!o) return fail(FV2D_ERR_ARG, "null output");
    const fv2d::HostMesh& m = h->s->mesh_;
    o[0] = m.np; o[1] = m.nf; o[2] = m.nc; o[3] = m.numBC1; o[4] = m.numBC2; o[5] = m.numWALL;
    o[6] = m.num_of_BC; o[7] = h->s->current_stage();
    return FV2D_OK;
}

int fv2d_save(fv2d_handle* h, int ndx) {
    NvtxRange nvtx_("fv2d_save");
    FV2D_H(h);
    const int N = h->s->mesh_.nc;
    std::vector<double> q(4 * (size_t)N), g(8 * (size_t)N), r(4 * (size_t)N);
    int rc = h->s->get_field(FV2D_F_QBAR, q.data());
    if (!rc) rc = h->s->get_field(FV2D_F_QBAR_GRAD, g.data());
    if (!rc) rc = h->s->get_field(FV2D_F_RES, r.data());
    if (rc && rc != FV2D_ERR_STATE) return fail(rc, h->s->err_);
    std::string err;
    int wrc = fv2d::save_solution(h->s->mesh_, h->cs, ndx, q.data(), g.data(), r.data(), "sol", err);
    if (wrc) return fail(wrc, err);
    return rc;
}

int fv2d_post(fv2d_handle* h, int ndx) {
    FV2D_H(h);
    std::vector<double> q(4 * (size_t)h->s->mesh_.nc);
    int rc = h->s->get_field(FV2D_F_QBAR, q.data());
    if (rc && rc != FV2D_ERR_STATE) return fail(rc, h->s->err_);
    std::string err;
    int wrc = fv2d::write_restart(h->s->mesh_, ndx, q.data(), "sol", err);
    if (wrc) return fail(wrc, err);
    return rc;
}

int fv2d_write_restart(fv2d_handle* h, const char* path, int ndx, int digits) {
    FV2D_H(h);
    if (!path || digits < 0 || digits > 17) return fail(FV2D_ERR_ARG, "bad argument");
    std::vector<double> q(4 * (size_t)h->s->mesh_.nc);
    int rc = h->s->get_field(FV2D_F_QBAR, q.data());
    if (rc && rc != FV2D_ERR_STATE) return fail(rc, h->s->err_);
    std::string err;
    int wrc = fv2d::write_restart_file(h->s->mesh_, path, ndx, q.data(), digits, err);
    if (wrc) return fail(wrc, err);
    return rc;
}

int fv2d_write_history_headers(fv2d_handle* h) {
    FV2D_H(h);
    std::string err;
    int rc = fv2d::write_history_headers("sol", err);
    return rc ? fail(rc, err) : FV2D_OK;
}

int fv2d_write_mesh_files(fv2d_handle* h) {
    FV2D_H(h);
    std::string err;
    int rc = fv2d::write_mesh_files(h->s->mesh_, "mesh", err);
    return rc ? fail(rc, err) : FV2D_OK;
}

int fv2d_read_restart(const char* path, int num_cells, int* ndx, double* q) {
    if (!path || !ndx || !q || num_cells <= 0) return fail(FV2D_ERR_ARG, "bad argument");
    std::string err;
    int rc = fv2d::read_restart(path, num_cells, ndx, q, err);
    return rc ? fail(rc, err) : FV2D_OK;
}

int fv2d_synchronize(fv2d_handle* h) { FV2D_H(h); FV2D_RET(h, h->s->synchronize()); }
int fv2d_set_store_residual(fv2d_handle* h, int every) { FV2D_H(h); FV2D_RET(h, h->s->set_store_residual(every)); }
int fv2d_set_graphs(fv2d_handle* h, int enable) { FV2D_H(h); FV2D_RET(h, h->s->set_graphs(enable)); }
int fv2d_set_kernel_timing(fv2d_handle* h, int enable) { FV2D_H(h); FV2D_RET(h, h->s->set_timing(enable)); }

int fv2d_kernel_times(fv2d_handle* h, char* names, int names_len, double* ms, int* launches, int max_kernels, int* n_kernels) {
    FV2D_H(h);
    double t[fv2d::K_COUNT];
    int l[fv2d::K_COUNT];
    int rc = h->s->kernel_times(t, l);
    if (rc) return fail(rc, h->s->err_);
    const int n = max_kernels < fv2d::K_COUNT ? max_kernels : fv2d::K_COUNT;
    std::string all;
    for (int i = 0; i < n; i++) {
        if (ms) ms[i] = t[i];
        if (launches) launches[i] = l[i];
        if (i) all += ",";
        all += fv2d::kKernelNames[i];
    }
    if (names && names_len > 0) std::snprintf(names, names_len, "%s", all.c_str());
    if (n_kernels) *n_kernels = n;
    return FV2D_OK;
}

void* fv2d_stream(fv2d_handle* h) { return (h && h->s) ? h->s->stream() : nullptr; }
long long fv2d_device_bytes(fv2d_handle* h) { return (h && h->s) ? h->s->device_bytes() : 0; }

const char* fv2d_last_error(fv2d_handle* h) {
    if (h && h->s && !h->s->err_.empty()) return h->s->err_.c_str();
    return g_err.c_str();
}


// ---- batch -------------------------------------------------------------------------------------
#define FV2D_BH(b) if (!(b) || !(b)->b) return fail(FV2D_ERR_ARG, "null batch")
#define FV2D_BRET(b, expr) do { int rc_ = (expr); if (rc_) g_err = (b)->b->err_; return rc_; } while (0)

int fv2d_batch_create(long long max_cells, long long max_faces, int max_solves, int precision, fv2d_batch** out) {
    if (!out) return fail(FV2D_ERR_ARG, "null output");
    *out = nullptr;
    if (precision != FV2D_FP64 && precision != FV2D_FP32) return fail(FV2D_ERR_ARG, "precision must be FV2D_FP64 or FV2D_FP32");
    int rc = check_device();
    if (rc) return rc;
    auto b = std::make_unique<fv2d_batch>();
    b->precision = precision;
    b->b.reset(precision == FV2D_FP64 ? fv2d::make_batch_fp64() : fv2d::make_batch_fp32());
    rc = b->b->init(max_cells, max_faces, max_solves);
    if (rc) return fail(rc, b->b->err_);
    *out = b.release();
    return FV2D_OK;
}

void fv2d_batch_destroy(fv2d_batch* b) { delete b; }

int fv2d_batch_footprint(const fv2d_mesh_desc* d, int precision, long long* bytes) {
    if (!d || !bytes) return fail(FV2D_ERR_ARG, "null argument");
    if (!d->face_cell2 || d->num_faces <= 0 || d->num_cells <= 0) return fail(FV2D_ERR_ARG, "empty mesh");
    long long nb = 0;
    for (int f = 0; f < d->num_faces; f++) nb += d->face_cell2[f] <= 0;
    fv2d::batch_footprint(precision, d->num_cells, d->num_faces, 2LL * d->num_faces - nb, bytes);
    return FV2D_OK;
}

int fv2d_batch_add(fv2d_batch* b, const fv2d_mesh_desc* desc, const fv2d_case* cs, int* solve_id) {
    NvtxRange nvtx_("fv2d_batch_add");
    FV2D_BH(b);
    if (!solve_id) return fail(FV2D_ERR_ARG, "null output");
    int rc = check_case(cs);
    if (rc) return rc;
    FV2D_BRET(b, b->b->add(desc, cs, solve_id));
}

int fv2d_batch_add_mesh(fv2d_batch* b, const fv2d_mesh* mesh, const fv2d_case* cs, int* solve_id) {
    NvtxRange nvtx_("fv2d_batch_add_mesh");
    FV2D_BH(b);
    if (!mesh || !solve_id) return fail(FV2D_ERR_ARG, "null argument");
    int rc = check_case(cs);
    if (rc) return rc;
    FV2D_BRET(b, b->b->add_mesh(mesh->m, cs, solve_id));
}

int fv2d_batch_remove(fv2d_batch* b, int solve_id) { FV2D_BH(b); FV2D_BRET(b, b->b->remove(solve_id)); }
int fv2d_batch_step(fv2d_batch* b, int iterations) { NvtxRange r("fv2d_batch_step"); FV2D_BH(b); FV2D_BRET(b, b->b->step(iterations)); }

int fv2d_batch_norms(fv2d_batch* b, int* ids, double* norms4, int* iterations, int max, int* n) {
    FV2D_BH(b);
    if (!ids || !norms4 || !n) return fail(FV2D_ERR_ARG, "null output");
    FV2D_BRET(b, b->b->norms(ids, norms4, iterations, max, n));
}

int fv2d_batch_get_state(fv2d_batch* b, int solve_id, double* q) {
    FV2D_BH(b);
    if (!q) return fail(FV2D_ERR_ARG, "null output");
    FV2D_BRET(b, b->b->get_state(solve_id, q));
}

int fv2d_batch_synchronize(fv2d_batch* b) { FV2D_BH(b); FV2D_BRET(b, b->b->synchronize()); }

int fv2d_batch_set_tuning(fv2d_batch* b, int block, const int* tile_mult3, const int* bucket_edges2) {
    FV2D_BH(b);
    fv2d::BatchTuning t = b->b->tuning();
    t.block = block;
    if (tile_mult3) for (int i = 0; i < 3; i++) t.tile_mult[i] = tile_mult3[i];
    if (bucket_edges2) for (int i = 0; i < 2; i++) t.bucket_edges[i] = bucket_edges2[i];
    FV2D_BRET(b, b->b->set_tuning(t));
}

int fv2d_batch_get_tuning(fv2d_batch* b, int* block, int* tile_mult3, int* bucket_edges2) {
    FV2D_BH(b);
    const fv2d::BatchTuning t = b->b->tuning();
    if (block) *block = t.block;
    if (tile_mult3) for (int i = 0; i < 3; i++) tile_mult3[i] = t.tile_mult[i];
    if (bucket_edges2) for (int i = 0; i < 2; i++) bucket_edges2[i] = t.bucket_edges[i];
    return FV2D_OK;
}

int fv2d_batch_set_grid_mode(fv2d_batch* b, int full_grid) {
    FV2D_BH(b);
    fv2d::BatchTuning t = b->b->tuning();
    t.full_grid = full_grid != 0;
    FV2D_BRET(b, b->b->set_tuning(t));
}

int fv2d_batch_usage(fv2d_batch* b, long long* out8) {
    FV2D_BH(b);
    if (!out8) return fail(FV2D_ERR_ARG, "null output");
    FV2D_BRET(b, b->b->usage(out8));
}

int fv2d_batch_set_kernel_timing(fv2d_batch* b, int enable) { FV2D_BH(b); FV2D_BRET(b, b->b->set_timing(enable)); }

int fv2d_batch_kernel_times(fv2d_batch* b, double* ms3, int* launches3) {
    FV2D_BH(b);
    if (!ms3 || !launches3) return fail(FV2D_ERR_ARG, "null output");
    FV2D_BRET(b, b->b->kernel_times(ms3, launches3));
}

void* fv2d_batch_stream(fv2d_batch* b) { return (b && b->b) ? b->b->stream() : nullptr; }

}  // extern "C"

namespace fv2d {
void batch_footprint(int precision, long long cells, long long faces, long long incs, long long* bytes) {
    if (precision == FV2D_FP32) { tiled_footprint(cells, faces, bytes); return; }
    const long long s = precision == FV2D_FP64 ? 8 : 4;
    const long long cell = (precision == FV2D_FP64 ? 9 : 11) * 4 * s + 4 * s + 24 + 4;   // Q[3], G[3], (D, lo), dt, S, vol, 1/vol, LSQ, offsets
    const long long face = 3 * 4 + 15 * s + 4 * s + s         // ids, geometry (+ 1/|dist|), contribution, spectral term
                           + (precision == FV2D_FP64 ? 8 * s : 0);   // FP64: stored face states (both sides)
    *bytes = (cells + 1) * cell + faces * face + incs * (8 + 4 * s);
}
}  // namespace fv2d
