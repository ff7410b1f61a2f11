/*
 * Reference harness -- TEST INFRASTRUCTURE ONLY.
 *
 * Builds the reference's own, unmodified sources (compiled in place from the reference tree by
 * oracle/Makefile; nothing is copied into this repository) and drives them through the
 * fv2d_oracle.h interface with prefix fvr_.  Setup restates src/base/main.cpp:49-118.  Two ways to
 * advance the solution:
 *   fvr_iterate : calls the reference ssp_rk3() (src/solver/ssp_rk3.cpp:18) n times;
 *   fvr_stage   : one RK stage, calling the reference res() (src/solver/res.cpp:21) and restating
 *                 the time-step and stage-combination loops of ssp_rk3.cpp:24-77, so per-stage
 *                 states can be read.  A test checks that three fvr_stage calls equal one
 *                 fvr_iterate call bit for bit.
 * The reference prints to std::cout; its output is discarded while it runs.
 */
#define main fv2d_reference_main
#include "src/base/main.cpp"
#undef main

#include "src/include/res.hpp"

#include <chrono>
#include <sstream>

#include "fv2d_oracle.h"

namespace {

struct Quiet {
    std::ostringstream sink;
    std::streambuf* old;
    Quiet() { old = std::cout.rdbuf(sink.rdbuf()); }
    ~Quiet() { std::cout.rdbuf(old); }
};

struct Ref {
    class_mesh mesh;
    class_Q Qbar, Qface, Qface_c1, Qface_c2, Qstar;
    class_flow freestream;
    class_residual residual;
    struct_size size;
    struct_inputs inputs;
    struct_BC BC;
    struct_time time;
    struct_report report;
    std::vector<double> dt;
    int stage = 0;
    bool have_qstar = false;
};

void stage_dt(Ref& r) {
    /* ssp_rk3.cpp:24-47 */
    const int N = r.size.num_cells;
    r.dt.assign(N, 0);
    for (int f = 0; f < r.size.num_faces; f++) {
        int c1 = r.mesh.face_cell1[f], c2 = r.mesh.face_cell2[f];
        r.dt[c1] += (std::abs(r.Qface_c1.Vn_avg[f]) + r.Qface_c1.c_avg[f]) * r.mesh.face_area[f];
        if (c2 >= 0) r.dt[c2] += (std::abs(r.Qface_c2.Vn_avg[f]) + r.Qface_c2.c_avg[f]) * r.mesh.face_area[f];
    }
    if (r.time.type == 1) {
        double mx = *std::max_element(r.dt.begin(), r.dt.end());
        for (int c = 0; c < N; c++) r.dt[c] = (2 * r.time.CFL * r.mesh.cell_vol[c]) / mx;
    } else if (r.time.type == 2) {
        for (int c = 0; c < N; c++) r.dt[c] = (2 * r.time.CFL * r.mesh.cell_vol[c]) / r.dt[c];
    }
}

void do_stage(Ref& r) {
    const int N = r.size.num_cells;
    class_Q& Qs = r.Qstar;
    std::vector<double>* qb[4] = {&r.Qbar.p1, &r.Qbar.p2, &r.Qbar.p3, &r.Qbar.p4};
    std::vector<double>* qs[4] = {&Qs.p1, &Qs.p2, &Qs.p3, &Qs.p4};
    std::vector<double>* rr[4] = {&r.residual.p1, &r.residual.p2, &r.residual.p3, &r.residual.p4};
    Quiet q;
    if (r.stage == 0) {
        Qs = class_Q();
        Qs.init(N, r.freestream.gamma, r.freestream.R);
        r.have_qstar = true;
        stage_dt(r);
        res(&r.residual, &r.mesh, &r.size, &r.inputs, &r.Qbar, &r.Qface, &r.Qface_c1, &r.Qface_c2, &r.freestream, &r.BC);
        for (int c = 0; c < N; c++)
            for (int k = 0; k < 4; k++) (*qs[k])[c] = (*qb[k])[c] + r.dt[c] * (*rr[k])[c];
        Qs.updateflow();
    } else if (r.stage == 1) {
        res(&r.residual, &r.mesh, &r.size, &r.inputs, &Qs, &r.Qface, &r.Qface_c1, &r.Qface_c2, &r.freestream, &r.BC);
        for (int c = 0; c < N; c++)
            for (int k = 0; k < 4; k++)
                (*qs[k])[c] = 0.75 * (*qb[k])[c] + 0.25 * (*qs[k])[c] + 0.25 * r.dt[c] * (*rr[k])[c];
        Qs.updateflow();
    } else {
        res(&r.residual, &r.mesh, &r.size, &r.inputs, &Qs, &r.Qface, &r.Qface_c1, &r.Qface_c2, &r.freestream, &r.BC);
        for (int c = 0; c < N; c++)
            for (int k = 0; k < 4; k++)
                (*qb[k])[c] = (1.0 / 3.0) * (*qb[k])[c] + (2.0 / 3.0) * (*qs[k])[c] + (2.0 / 3.0) * r.dt[c] * (*rr[k])[c];
        r.Qbar.updateflow();
    }
    r.stage = (r.stage + 1) % 3;
}

int put(const std::vector<double>& a, double* out, int off) {
    std::copy(a.begin(), a.end(), out + off);
    return off + (int)a.size();
}

}  // namespace

extern "C" {

void* fvr_open(const char* input_file) {
    Ref* r = new Ref();
    Quiet q;
    char arg0[] = "fv2d";
    std::string a1 = input_file;
    char* argv[3] = {arg0, &a1[0], nullptr};
    r->size.numWALL = -1;
    {
        std::ifstream probe(input_file);
        if (!probe.is_open()) { delete r; return nullptr; }
    }
    read_inputs(&r->freestream, &r->inputs, &r->BC, &r->time, &r->report, 2, argv);  /* main.cpp:56 */
    {
        std::ifstream probe(r->inputs.grid_file);
        if (!probe.is_open()) { delete r; return nullptr; }
    }
    readmesh(&r->mesh, r->inputs.grid_file, &r->size, &r->BC, &r->inputs);           /* main.cpp:57 */
    r->freestream.update_vis();                                                      /* main.cpp:77-80 */
    r->freestream.updateQ();
    r->freestream.free_comp();
    r->residual.init(r->size.num_cells);
    r->Qbar.init(r->size.num_cells, &r->freestream);                                 /* main.cpp:108-109 */
    r->Qbar.updateQ();
    if (r->inputs.eqn == 2) r->Qface.init(r->size.num_faces, &r->freestream);        /* main.cpp:114-118 */
    r->Qface_c1.init(r->size.num_faces, &r->freestream);
    r->Qface_c2.init(r->size.num_faces, &r->freestream);
    return r;
}

void fvr_close(void* h) { delete (Ref*)h; }

void fvr_sizes(void* h, int* out) {
    Ref* r = (Ref*)h;
    out[0] = r->size.num_points; out[1] = r->size.num_faces; out[2] = r->size.num_cells;
    out[3] = r->size.numBC1; out[4] = r->size.numBC2; out[5] = r->size.numWALL;
    out[6] = r->mesh.num_of_BC; out[7] = r->stage;
}

void fvr_stage(void* h) { do_stage(*(Ref*)h); }

void fvr_iterate(void* h, int n) {
    Ref* r = (Ref*)h;
    Quiet q;
    for (int i = 0; i < n; i++)                                                      /* main.cpp:121-133 */
        ssp_rk3(&r->mesh, &r->Qbar, &r->Qface, &r->Qface_c1, &r->Qface_c2, &r->residual, &r->size,
                &r->inputs, &r->freestream, &r->BC, &r->time);
}

double fvr_time_iterations(void* h, int n) {
    auto t0 = std::chrono::steady_clock::now();
    fvr_iterate(h, n);
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

void fvr_set_state(void* h, const double* qv) {
    /* restart path, main.cpp:94-106 (with fresh face states, main.cpp:114-118) */
    Ref* r = (Ref*)h;
    const int N = r->size.num_cells;
    if (r->inputs.eqn == 2) r->Qface.init(r->size.num_faces, &r->freestream);
    r->Qface_c1.init(r->size.num_faces, &r->freestream);
    r->Qface_c2.init(r->size.num_faces, &r->freestream);
    r->Qbar.init(N, r->freestream.gamma, r->freestream.R);
    for (int c = 0; c < N; c++) {
        r->Qbar.p1[c] = qv[c]; r->Qbar.p2[c] = qv[N + c]; r->Qbar.p3[c] = qv[2 * N + c]; r->Qbar.p4[c] = qv[3 * N + c];
    }
    r->Qbar.updateflow();
    r->stage = 0;
}

int fvr_get(void* h, int field, double* out) {
    Ref* r = (Ref*)h;
    class_mesh& m = r->mesh;
    int n = 0;
    switch (field) {
        case FVO_QBAR: n = put(r->Qbar.p1, out, 0); n = put(r->Qbar.p2, out, n); n = put(r->Qbar.p3, out, n); n = put(r->Qbar.p4, out, n); break;
        case FVO_QSTAR: if (!r->have_qstar) return -1;
            n = put(r->Qstar.p1, out, 0); n = put(r->Qstar.p2, out, n); n = put(r->Qstar.p3, out, n); n = put(r->Qstar.p4, out, n); break;
        case FVO_RES: n = put(r->residual.p1, out, 0); n = put(r->residual.p2, out, n); n = put(r->residual.p3, out, n); n = put(r->residual.p4, out, n); break;
        case FVO_DT: if (r->dt.empty()) return -1; n = put(r->dt, out, 0); break;
        case FVO_QBAR_GRAD: case FVO_QSTAR_GRAD: {
            if (field == FVO_QSTAR_GRAD && !r->have_qstar) return -1;
            class_Q& s = (field == FVO_QBAR_GRAD) ? r->Qbar : r->Qstar;
            for (std::vector<double>* a : {&s.Qxp1, &s.Qxp2, &s.Qxp3, &s.Qxp4, &s.Qyp1, &s.Qyp2, &s.Qyp3, &s.Qyp4}) n = put(*a, out, n);
            break;
        }
        case FVO_QF1: n = put(r->Qface_c1.p1, out, 0); n = put(r->Qface_c1.p2, out, n); n = put(r->Qface_c1.p3, out, n); n = put(r->Qface_c1.p4, out, n); break;
        case FVO_QF2: n = put(r->Qface_c2.p1, out, 0); n = put(r->Qface_c2.p2, out, n); n = put(r->Qface_c2.p3, out, n); n = put(r->Qface_c2.p4, out, n); break;
        case FVO_VNC: n = put(r->Qface_c1.Vn_avg, out, 0); n = put(r->Qface_c1.c_avg, out, n); break;
        case FVO_QBAR_PRIM: n = put(r->Qbar.rho, out, 0); n = put(r->Qbar.u, out, n); n = put(r->Qbar.v, out, n); n = put(r->Qbar.P, out, n); break;
        case FVO_G_AREA: n = put(m.face_area, out, 0); break;
        case FVO_G_NX: n = put(m.face_nx, out, 0); break;
        case FVO_G_NY: n = put(m.face_ny, out, 0); break;
        case FVO_G_FCX: n = put(m.face_centerx, out, 0); break;
        case FVO_G_FCY: n = put(m.face_centery, out, 0); break;
        case FVO_G_C1DX: n = put(m.face_cell1_dx, out, 0); break;
        case FVO_G_C1DY: n = put(m.face_cell1_dy, out, 0); break;
        case FVO_G_C2DX: n = put(m.face_cell2_dx, out, 0); break;
        case FVO_G_C2DY: n = put(m.face_cell2_dy, out, 0); break;
        case FVO_G_DXJ: n = put(m.face_dxj, out, 0); break;
        case FVO_G_DYJ: n = put(m.face_dyj, out, 0); break;
        case FVO_G_DIST: n = put(m.face_dist, out, 0); break;
        case FVO_G_LX: n = put(m.face_lx, out, 0); break;
        case FVO_G_LY: n = put(m.face_ly, out, 0); break;
        case FVO_G_MX: n = put(m.face_mx, out, 0); break;
        case FVO_G_MY: n = put(m.face_my, out, 0); break;
        case FVO_G_VOL: n = put(m.cell_vol, out, 0); break;
        case FVO_G_CCX: n = put(m.cell_centerx, out, 0); break;
        case FVO_G_CCY: n = put(m.cell_centery, out, 0); break;
        case FVO_G_IXX: n = put(m.Ixx, out, 0); break;
        case FVO_G_IYY: n = put(m.Iyy, out, 0); break;
        case FVO_G_IXY: n = put(m.Ixy, out, 0); break;
        case FVO_G_DELTA: n = put(m.delta, out, 0); break;
        case FVO_G_BCCX: n = put(m.BC_cell_centerx, out, 0); break;
        case FVO_G_BCCY: n = put(m.BC_cell_centery, out, 0); break;
        default: return -1;
    }
    return n;
}

int fvr_get_int(void* h, int field, int* out) {
    Ref* r = (Ref*)h;
    class_mesh& m = r->mesh;
    switch (field) {
        case FVO_I_FC1: std::copy(m.face_cell1.begin(), m.face_cell1.end(), out); return (int)m.face_cell1.size();
        case FVO_I_FC2: std::copy(m.face_cell2.begin(), m.face_cell2.end(), out); return (int)m.face_cell2.size();
        case FVO_I_FP1: std::copy(m.face_point1.begin(), m.face_point1.end(), out); return (int)m.face_point1.size();
        case FVO_I_FP2: std::copy(m.face_point2.begin(), m.face_point2.end(), out); return (int)m.face_point2.size();
        case FVO_I_CFC: std::copy(m.cell_face_count.begin(), m.cell_face_count.end(), out); return (int)m.cell_face_count.size();
        case FVO_I_BCF: for (size_t i = 0; i < m.BC_faces.size(); i++) out[i] = (int)m.BC_faces[i]; return (int)m.BC_faces.size();
        default: return -1;
    }
}

}  // extern "C"
