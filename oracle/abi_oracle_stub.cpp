/*
 * TEST INFRASTRUCTURE ONLY: the few C-ABI entry points the reference-signature shim
 * (cfd-2d-ns-fv_gb300/shim/ssp_rk3_gpu.cpp) calls, implemented on the ORACLE PORT instead of the
 * GPU.  Linking the reference's own src/base/main.cpp with the shim and this file gives a CPU
 * program whose output files must equal the reference program's; that checks the shim's
 * marshalling (mesh and option conversion, fresh/restart detection, what it copies back into the
 * caller's objects) where no GPU exists.  The product library never contains this file.
 */
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fv2d_gpu.h"
#include "fv2d_oracle.h"

struct fv2d_handle {
    void* o = nullptr;
    int nc = 0;
};

static std::string g_err = "oracle stub";

extern "C" {

int fv2d_create(const fv2d_mesh_desc* d, const fv2d_case* cs, int precision, fv2d_handle** out) {
    if (!d || !cs || !out || precision != FV2D_FP64) { g_err = "oracle stub: bad argument"; return FV2D_ERR_ARG; }
    fvo_case c;
    c.order = cs->order; c.eqn = cs->eqn; c.flux_solver = cs->flux_solver; c.limiter = cs->limiter;
    c.time_type = cs->time_type; c.time_scheme = cs->time_scheme; c.bc1 = cs->bc1; c.bc2 = cs->bc2;
    c.cfl = cs->cfl; c.gamma = cs->gamma; c.R = cs->R; c.mu = cs->mu; c.Pr = cs->Pr;
    c.P = cs->P; c.rho = cs->rho; c.u = cs->u; c.v = cs->v;
    void* o = fvo_open_arrays(&c, d->num_points, d->num_faces, d->num_cells, d->x, d->y, d->face_point1,
                              d->face_point2, d->face_cell1, d->face_cell2);
    if (!o) { g_err = "oracle stub: cannot open"; return FV2D_ERR_MESH; }
    *out = new fv2d_handle{o, d->num_cells};
    return FV2D_OK;
}

void fv2d_destroy(fv2d_handle* h) {
    if (h) fvo_close(h->o);
    delete h;
}

int fv2d_step(fv2d_handle* h, int iterations) {
    fvo_iterate(h->o, iterations);
    return FV2D_OK;
}

int fv2d_get_state(fv2d_handle* h, double* q) { return fvo_get(h->o, FVO_QBAR, q) < 0 ? FV2D_ERR_ARG : FV2D_OK; }

int fv2d_get_field(fv2d_handle* h, int field, double* out) {
    return fvo_get(h->o, field, out) < 0 ? FV2D_ERR_ARG : FV2D_OK;   // field ids shared with the oracle
}

int fv2d_set_state(fv2d_handle* h, const double* q) {
    fvo_set_state(h->o, q);
    return FV2D_OK;
}

int fv2d_load_state(fv2d_handle*, const double*) {
    g_err = "oracle stub: load_state is not available";
    return FV2D_ERR_ARG;
}

const char* fv2d_last_error(fv2d_handle*) { return g_err.c_str(); }

}  // extern "C"
