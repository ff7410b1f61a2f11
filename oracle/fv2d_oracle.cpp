/*
 * fv2d oracle port -- TEST INFRASTRUCTURE ONLY (the oracle; never linked into the product).
 *
 * A plain, single-threaded CPU restatement of the reference solver step of
 * Avery-Hantla/CFD-2D-NS-FV (fv2d): input parsing, grid reading + geometry, LSQ gradient, squeeze
 * limiter, reconstruction + boundary conditions, NS face terms, Rusanov flux, residual assembly,
 * time step and SSP-RK3 stages.  Every loop visits faces and cells in the reference's order and
 * every floating-point expression keeps the reference's operation order, so that (compiled with
 * -ffp-contract=off) its FP64 results are bit-identical to the reference on every mesh the
 * reference can read.  Unlike the reference, cells keep variable-length face lists (CSR), so
 * meshes with 7-9-sided cells (which overflow the reference's 6 slots, src/base/readmesh.cpp:38)
 * are handled.  Out-of-bounds reads of the reference whose results are discarded are skipped.
 *
 * Citations are file:line in the reference project.
 */
#include "fv2d_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <string>
#include <vector>

namespace {

typedef std::vector<double> vd;
typedef std::vector<int> vi;

/* class_flow (src/support/class_flow.hpp:3-46) */
struct Flow {
    double gamma = 0, P = 0, rho = 0, u = 0, v = 0, E = 0;
    double Q1 = 0, Q2 = 0, Q3 = 0, Q4 = 0;
    double R = 0, mu = 0, Pr = 0, Cp = 0, T = 0, k = 0;
    double flowx = 0, flowy = 0;
    void updateQ() {                                   /* class_flow.hpp:28-34 */
        Q1 = rho;
        Q2 = rho * u;
        Q3 = rho * v;
        E = (P / (gamma - 1)) + 0.5 * rho * (u * u + v * v);
        Q4 = E;
    }
    void update_vis() {                                /* class_flow.hpp:36-40 */
        Cp = R * gamma / (gamma - 1);
        T = P / (rho * R);
        k = (mu * Cp) / Pr;
    }
    void free_comp() {                                 /* class_flow.hpp:42-46 */
        double norm = std::sqrt(u * u + v * v);
        flowx = u / norm;
        flowy = v / norm;
    }
};

/* class_Q (src/support/class_q.hpp:6-173) */
struct State {
    double R = 0, gamma = 0, k = 0, mu = 0;
    vd p1, p2, p3, p4, rho, u, v, E, P, c, T, Vn_avg, c_avg;
    vd Qxp1, Qxp2, Qxp3, Qxp4, Qyp1, Qyp2, Qyp3, Qyp4;
    vd tau_xx, tau_xy, tau_yy, dTdx, dTdy;

    void init(int n, const Flow& f) {                  /* class_q.hpp:50-94 */
        gamma = f.gamma; R = f.R; mu = f.mu; k = f.k;
        P.assign(n, f.P); rho.assign(n, f.rho); u.assign(n, f.u); v.assign(n, f.v);
        Vn_avg.assign(n, std::sqrt(f.v * f.v + f.u * f.u));
        c_avg.assign(n, std::sqrt(gamma * (f.P / f.rho)));
        E.assign(n, -101); c.assign(n, -101); T.assign(n, -101);
        for (int i = 0; i < n; i++) {
            E[i] = (P[i] / (gamma - 1)) + 0.5 * rho[i] * (u[i] * u[i] + v[i] * v[i]);
            c[i] = std::sqrt(gamma * (P[i] / rho[i]));
            T[i] = P[i] / (rho[i] * R);
        }
        p1.assign(n, -101); p2.assign(n, -101); p3.assign(n, -101); p4.assign(n, -101);
        for (vd* g : {&Qxp1, &Qxp2, &Qxp3, &Qxp4, &Qyp1, &Qyp2, &Qyp3, &Qyp4}) g->assign(n, 0);
        tau_xx.assign(n, 0); tau_xy.assign(n, 0); tau_yy.assign(n, 0);
        dTdx.assign(n, 0); dTdy.assign(n, 0);
    }
    void init(int n, double g, double r) {             /* class_q.hpp:96-129 (mu, k left unset) */
        gamma = g; R = r;
        for (vd* a : {&P, &rho, &u, &v, &E, &c, &T, &p1, &p2, &p3, &p4, &Vn_avg, &c_avg}) a->assign(n, -101);
        for (vd* a : {&Qxp1, &Qxp2, &Qxp3, &Qxp4, &Qyp1, &Qyp2, &Qyp3, &Qyp4}) a->assign(n, 0);
    }
    void updateflow() {                                /* class_q.hpp:131-141 */
        rho = p1;
        E = p4;
        for (size_t i = 0; i < p1.size(); i++) {
            u[i] = p2[i] / rho[i];
            v[i] = p3[i] / rho[i];
            P[i] = (E[i] - (0.5 * rho[i] * (u[i] * u[i] + v[i] * v[i]))) * (gamma - 1);
            c[i] = std::sqrt(gamma * (P[i] / rho[i]));
            T[i] = P[i] / (rho[i] * R);
        }
    }
    void updateflow_int(int i) {                       /* class_q.hpp:143-151 */
        rho[i] = p1[i];
        E[i] = p4[i];
        u[i] = p2[i] / rho[i];
        v[i] = p3[i] / rho[i];
        P[i] = (E[i] - (0.5 * rho[i] * (u[i] * u[i] + v[i] * v[i]))) * (gamma - 1);
        c[i] = std::sqrt(gamma * (P[i] / rho[i]));
        T[i] = P[i] / (rho[i] * R);
    }
    void updateQ() {                                   /* class_q.hpp:153-161 */
        p1 = rho;
        for (size_t i = 0; i < p1.size(); i++) {
            p2[i] = rho[i] * u[i];
            p3[i] = rho[i] * v[i];
            E[i] = (P[i] / (gamma - 1)) + 0.5 * rho[i] * (u[i] * u[i] + v[i] * v[i]);
        }
        p4 = E;
    }
    void comp_vis(int i, double ux, double uy, double vx, double vy,
                  double Px, double Py, double rhox, double rhoy) {   /* class_q.hpp:163-169 */
        tau_xx[i] = 2 * mu * (ux - (ux + vy) / 3);
        tau_xy[i] = mu * (uy + vx);
        tau_yy[i] = 2 * mu * (vy - (ux + vy) / 3);
        dTdx[i] = (Px * rho[i] - rhox * P[i]) / (R * rho[i] * rho[i]);
        dTdy[i] = (Py * rho[i] - rhoy * P[i]) / (R * rho[i] * rho[i]);
    }
};

struct Mesh {
    int np = 0, nf = 0, nc = 0;
    int numBC1 = 0, numBC2 = 0, numWALL = -1, num_of_BC = 0;
    vd x, y;
    vi fp1, fp2, fc1, fc2;
    vi cf_off, cf;                  /* CSR cell -> faces, in face-read (ascending) order */
    vi cf_count;
    vi BC_faces, face2BCf;
    vd area, nx, ny, fcx, fcy, vol, ccx, ccy, bccx, bccy;
    vd c1dx, c1dy, c2dx, c2dy, dxj, dyj, delta, Ixx, Iyy, Ixy;
    vd dist, lx, ly, mx, my;
};

struct Case {
    int order = 0, nmax = 0, monitor_step = 0, output_step = 0, restart = 0;
    std::string grid_file;
    int eqn = 0, flux_solver = 0, limiter = 0;
    int scheme = 0, type = 0;
    double CFL = 0;
    double length = 0;
    int BC1 = 0, BC2 = 0;
};

struct Oracle {
    Case cs;
    Flow fs;
    Mesh m;
    State Qbar, Qface, Qface_c1, Qface_c2, Qstar;
    vd r1, r2, r3, r4;              /* class_residual */
    vd dt;
    int stage = 0;
    bool have_qstar = false;
};

/* ---------------------------------------------------------------- input.in
 * read_inputs (src/base/read_inputs.cpp:10-219): 9 section tokens, each followed by a fixed
 * number of "key = value" triples; string values map to integer codes.                        */
bool read_inputs(const char* path, Case& cs, Flow& fs) {
    std::ifstream in(path);
    if (!in.is_open()) return false;
    std::string s1, s2, eq;
    auto triples = [&](int n, auto&& fn) {
        for (int j = 0; j < n; j++) { in >> s1 >> eq >> s2; fn(); }
    };
    for (int sec = 0; sec < 9; sec++) {
        in >> s1;
        if (s1 == "[case]") triples(5, [&] {           /* read_inputs.cpp:23-31 */
            if (s1 == "solution_poly_order") cs.order = std::stoi(s2) + 1;
            if (s1 == "nmax") cs.nmax = std::stoi(s2);
            if (s1 == "monitor_step") cs.monitor_step = std::stoi(s2);
            if (s1 == "output_step") cs.output_step = std::stoi(s2);
            if (s1 == "restart") cs.restart = std::stoi(s2);
        });
        if (s1 == "[limiter]") triples(1, [&] {        /* read_inputs.cpp:40-58 */
            if (s1 == "limiter") {
                if (s2 == "NONE") cs.limiter = 0;
                if (s2 == "MINMOD") cs.limiter = 1;
                if (s2 == "SQUEEZE") cs.limiter = 2;
            }
        });
        if (s1 == "[grid]") triples(1, [&] {           /* read_inputs.cpp:61-65 */
            if (s1 == "grid_file") cs.grid_file = s2;
        });
        if (s1 == "[equations]") triples(2, [&] {      /* read_inputs.cpp:70-94 */
            if (s1 == "eqn") { if (s2 == "EULER") cs.eqn = 1; if (s2 == "NS") cs.eqn = 2; }
            if (s1 == "flux_solver") { if (s2 == "RUSANOV") cs.flux_solver = 1; if (s2 == "ROE") cs.flux_solver = 2; }
        });
        if (s1 == "[fluid]") triples(4, [&] {          /* read_inputs.cpp:97-104 */
            if (s1 == "gamma") fs.gamma = std::stod(s2);
            if (s1 == "R") fs.R = std::stod(s2);
            if (s1 == "mu") fs.mu = std::stod(s2);
            if (s1 == "Pr") fs.Pr = std::stod(s2);
        });
        if (s1 == "[init]") triples(4, [&] {           /* read_inputs.cpp:113-120 */
            if (s1 == "P") fs.P = std::stod(s2);
            if (s1 == "rho") fs.rho = std::stod(s2);
            if (s1 == "u") fs.u = std::stod(s2);
            if (s1 == "v") fs.v = std::stod(s2);
        });
        if (s1 == "[time]") triples(3, [&] {           /* read_inputs.cpp:128-154 */
            if (s1 == "CFL") cs.CFL = std::stod(s2);
            if (s1 == "time_step_type") { if (s2 == "GLOBAL") cs.type = 1; if (s2 == "LOCAL") cs.type = 2; }
            if (s1 == "time_scheme") { if (s2 == "SSP_RK2") cs.scheme = 1; if (s2 == "SSP_RK3") cs.scheme = 2; }
        });
        if (s1 == "[report]") triples(1, [&] {         /* read_inputs.cpp:158-162 */
            if (s1 == "length") cs.length = std::stod(s2);
        });
        if (s1 == "[BC]") triples(2, [&] {             /* read_inputs.cpp:167-207 */
            int* dst = (s1 == "BC1") ? &cs.BC1 : (s1 == "BC2") ? &cs.BC2 : nullptr;
            if (dst) {
                if (s2 == "FREESTREAM") *dst = -1;
                if (s2 == "SLIP_WALL") *dst = -2;
                if (s2 == "EXTRAPOLATION") *dst = -3;
                if (s2 == "NO_SLIP_WALL") *dst = -4;
            }
        });
    }
    return true;
}

/* ---------------------------------------------------------------- grid + geometry
 * Connectivity: readmesh.cpp:31-85 (file c2 == 0 -> BC1 code, c2 == -1 -> BC2 code; cell face
 * lists filled in face-read order).  Geometry: readmesh.cpp:117-411.                          */
void build_connectivity(Mesh& m, const Case& cs, const int* fp1, const int* fp2,
                        const int* fc1, const int* fc2) {
    m.fp1.resize(m.nf); m.fp2.resize(m.nf); m.fc1.resize(m.nf); m.fc2.resize(m.nf);
    m.face2BCf.assign(m.nf, -101);
    m.cf_count.assign(m.nc, 0);
    m.numBC1 = m.numBC2 = m.num_of_BC = 0;
    m.BC_faces.clear();
    for (int f = 0; f < m.nf; f++) {
        m.fp1[f] = fp1[f] - 1;
        m.fp2[f] = fp2[f] - 1;
        int i1 = fc1[f], i2 = fc2[f];
        m.fc1[f] = i1 - 1;
        if (i2 - 1 == -1) { m.fc2[f] = cs.BC1; m.numBC1++; }
        else if (i2 - 1 == -2) { m.fc2[f] = cs.BC2; m.numBC2++; }
        else m.fc2[f] = i2 - 1;
        m.cf_count[i1 - 1]++;
        if (i2 > 0) m.cf_count[i2 - 1]++;
        if (i2 - 1 < 0) { m.BC_faces.push_back(f); m.face2BCf[f] = m.num_of_BC; m.num_of_BC++; }
    }
    m.cf_off.assign(m.nc + 1, 0);
    for (int c = 0; c < m.nc; c++) m.cf_off[c + 1] = m.cf_off[c] + m.cf_count[c];
    m.cf.assign(m.cf_off[m.nc], -101);
    vi fill(m.nc, 0);
    for (int f = 0; f < m.nf; f++) {
        int c1 = fc1[f] - 1;
        m.cf[m.cf_off[c1] + fill[c1]++] = f;
        if (fc2[f] > 0) { int c2 = fc2[f] - 1; m.cf[m.cf_off[c2] + fill[c2]++] = f; }
    }
    /* readmesh.cpp:356-360: numWALL is left unset when neither BC is a wall */
    if (cs.BC1 == -2 || cs.BC1 == -4) m.numWALL = m.numBC1;
    else if (cs.BC2 == -2 || cs.BC2 == -4) m.numWALL = m.numBC2;
}

void build_geometry(Mesh& m) {
    const int nf = m.nf, nc = m.nc;
    m.area.resize(nf); m.nx.resize(nf); m.ny.resize(nf); m.fcx.resize(nf); m.fcy.resize(nf);
    for (int f = 0; f < nf; f++) {                     /* readmesh.cpp:117-139 */
        double x1 = m.x[m.fp1[f]], y1 = m.y[m.fp1[f]];
        double x2 = m.x[m.fp2[f]], y2 = m.y[m.fp2[f]];
        double dx = x2 - x1, dy = y2 - y1;
        double area = sqrt(dx * dx + dy * dy);
        m.area[f] = area;
        m.nx[f] = dy / area;
        m.ny[f] = -dx / area;
        m.fcx[f] = dx / 2 + x1;
        m.fcy[f] = dy / 2 + y1;
    }
    m.vol.resize(nc); m.ccx.resize(nc); m.ccy.resize(nc);
    vd px, py;
    for (int c = 0; c < nc; c++) {                     /* readmesh.cpp:147-228 */
        const int vc = m.cf_count[c];
        int found = 0;
        px.assign(vc, 0); py.assign(vc, 0);
        for (int j = m.cf_off[c]; j < m.cf_off[c + 1]; j++) {
            const int f = m.cf[j];
            double t1x = m.x[m.fp1[f]], t1y = m.y[m.fp1[f]];
            double t2x = m.x[m.fp2[f]], t2y = m.y[m.fp2[f]];
            bool f1 = false, f2 = false;
            for (int z = 0; z < vc; z++) if (px[z] == t1x && py[z] == t1y) { f1 = true; break; }
            if (!f1 && found < vc) { px[found] = t1x; py[found] = t1y; found++; }
            for (int z = 0; z < vc; z++) if (px[z] == t2x && py[z] == t2y) { f2 = true; break; }
            if (!f2 && found < vc) { px[found] = t2x; py[found] = t2y; found++; }
        }
        double sx = 0, sy = 0;
        for (int j = 0; j < vc; j++) { sx += px[j]; sy += py[j]; }
        const double cx = sx / vc, cy = sy / vc;
        double sum_vol = 0, scx = 0, scy = 0;
        for (int j = m.cf_off[c]; j < m.cf_off[c + 1]; j++) {
            const int f = m.cf[j];
            double x1x = m.x[m.fp1[f]], y1x = m.y[m.fp1[f]];
            double x2x = m.x[m.fp2[f]], y2x = m.y[m.fp2[f]];
            double x3x = cx, y3x = cy;
            double vs = 0.5 * std::abs(x1x * (y2x - y3x) + x2x * (y3x - y1x) + x3x * (y1x - y2x));
            sum_vol += vs;
            double csx = (x1x + x2x + x3x) / 3;
            double csy = (y1x + y2x + y3x) / 3;
            scx += csx * vs;
            scy += csy * vs;
        }
        m.vol[c] = sum_vol;
        m.ccx[c] = scx / sum_vol;
        m.ccy[c] = scy / sum_vol;
    }
    m.bccx.assign(m.num_of_BC, -101); m.bccy.assign(m.num_of_BC, -101);
    for (int i = 0; i < m.num_of_BC; i++) {            /* readmesh.cpp:235-244 */
        const int f = m.BC_faces[i];
        const int c1 = m.fc1[f];
        double rx = m.fcx[f] - m.ccx[c1];
        double ry = m.fcy[f] - m.ccy[c1];
        double nt = 2.0 * (rx * m.nx[f] + ry * m.ny[f]);
        m.bccx[i] = m.ccx[c1] + nt * m.nx[f];
        m.bccy[i] = m.ccy[c1] + nt * m.ny[f];
    }
    m.c1dx.assign(nf, -101); m.c1dy.assign(nf, -101); m.c2dx.assign(nf, -101); m.c2dy.assign(nf, -101);
    for (int f = 0; f < nf; f++) {                     /* readmesh.cpp:252-265 */
        m.c1dx[f] = m.fcx[f] - m.ccx[m.fc1[f]];
        m.c1dy[f] = m.fcy[f] - m.ccy[m.fc1[f]];
        if (m.fc2[f] >= 0) {
            m.c2dx[f] = m.fcx[f] - m.ccx[m.fc2[f]];
            m.c2dy[f] = m.fcy[f] - m.ccy[m.fc2[f]];
        } else {
            const int b = m.face2BCf[f];
            m.c2dx[f] = m.fcx[f] - m.bccx[b];
            m.c2dy[f] = m.fcy[f] - m.bccy[b];
        }
    }
    vd d1(nc, 0), d2(nc, 0), d3(nc, 0);
    m.dxj.assign(nf, -101); m.dyj.assign(nf, -101);
    for (int f = 0; f < nf; f++) {                     /* readmesh.cpp:278-306 */
        const int c1 = m.fc1[f], c2 = m.fc2[f];
        double xi = m.ccx[c1], yi = m.ccy[c1], xj, yj;
        if (c2 >= 0) { xj = m.ccx[c2]; yj = m.ccy[c2]; }
        else { const int b = m.face2BCf[f]; xj = m.bccx[b]; yj = m.bccy[b]; }
        d1[c1] += (xi - xj) * (xi - xj);
        d2[c1] += (yi - yj) * (yi - yj);
        d3[c1] += ((xi - xj) * (yi - yj));
        if (c2 >= 0) {
            d1[c2] += (xj - xi) * (xj - xi);
            d2[c2] += (yj - yi) * (yj - yi);
            d3[c2] += ((xj - xi) * (yj - yi));
        }
        m.dxj[f] = xj - xi;
        m.dyj[f] = yj - yi;
    }
    m.delta.resize(nc); m.Ixx.resize(nc); m.Iyy.resize(nc); m.Ixy.resize(nc);
    for (int c = 0; c < nc; c++) m.delta[c] = d1[c] * d2[c] - (d3[c] * d3[c]);   /* :308-310 */
    for (int c = 0; c < nc; c++) {                     /* readmesh.cpp:316-320 */
        m.Ixx[c] = d1[c] / m.delta[c];
        m.Iyy[c] = d2[c] / m.delta[c];
        m.Ixy[c] = d3[c] / m.delta[c];
    }
    /* readmesh.cpp:365-411.  For boundary faces the reference indexes BC_faces[] by the FACE id
     * (:373, :394); that is only in range (and only meaningful) when boundary faces come first.
     * Out-of-range lookups, which the reference performs as unchecked reads, give NaN here;
     * the solver never reads these values on boundary faces.                                   */
    const double qnan = std::numeric_limits<double>::quiet_NaN();
    m.dist.assign(nf, -101); m.lx.assign(nf, -101); m.ly.assign(nf, -101);
    m.mx.assign(nf, -101); m.my.assign(nf, -101);
    for (int f = 0; f < nf; f++) {
        const int c1 = m.fc1[f], c2 = m.fc2[f];
        double tx, ty;
        if (c2 >= 0) { tx = m.ccx[c2] - m.ccx[c1]; ty = m.ccy[c2] - m.ccy[c1]; }
        else if (f < m.num_of_BC && m.BC_faces[f] < m.num_of_BC) {
            const int b = m.BC_faces[f];
            tx = m.bccx[b] - m.ccx[c1]; ty = m.bccy[b] - m.ccy[c1];
        } else { tx = qnan; ty = qnan; }
        m.dist[f] = std::sqrt(tx * tx + ty * ty);
        m.lx[f] = tx; m.ly[f] = ty;
        m.mx[f] = (m.x[m.fp2[f]] - m.x[m.fp1[f]]);
        m.my[f] = (m.y[m.fp2[f]] - m.y[m.fp1[f]]);
        double t = std::sqrt(m.mx[f] * m.mx[f] + m.my[f] * m.my[f]);
        m.mx[f] = m.mx[f] / t;
        m.my[f] = m.my[f] / t;
        double t2 = std::sqrt(m.lx[f] * m.lx[f] + m.ly[f] * m.ly[f]);
        m.lx[f] = m.lx[f] / t2;
        m.ly[f] = m.ly[f] / t2;
    }
}

bool read_grid_file(const char* path, Mesh& m, vi& fp1, vi& fp2, vi& fc1, vi& fc2) {
    std::ifstream g(path);                             /* readmesh.cpp:21-108 */
    if (!g.is_open()) return false;
    g >> m.np >> m.nf >> m.nc;
    if (!g || m.np <= 0 || m.nf <= 0 || m.nc <= 0) return false;
    m.x.resize(m.np); m.y.resize(m.np);
    for (int i = 0; i < m.np; i++) g >> m.x[i] >> m.y[i];
    fp1.resize(m.nf); fp2.resize(m.nf); fc1.resize(m.nf); fc2.resize(m.nf);
    for (int f = 0; f < m.nf; f++) g >> fp1[f] >> fp2[f];
    for (int f = 0; f < m.nf; f++) g >> fc1[f] >> fc2[f];
    return (bool)g;
}

/* main.cpp:75-118: freestream, residual, Qbar (uniform freestream) and face states */
void setup(Oracle& o) {
    o.fs.update_vis();
    o.fs.updateQ();
    o.fs.free_comp();
    const int N = o.m.nc, F = o.m.nf;
    o.r1.assign(N, 0); o.r2.assign(N, 0); o.r3.assign(N, 0); o.r4.assign(N, 0);
    o.Qbar.init(N, o.fs);
    o.Qbar.updateQ();
    if (o.cs.eqn == 2) o.Qface.init(F, o.fs);
    o.Qface_c1.init(F, o.fs);
    o.Qface_c2.init(F, o.fs);
    o.dt.assign(N, 0);
    o.stage = 0;
}

/* ---------------------------------------------------------------- solver step */

/* compute_gradient (src/solver/cell_gradient.cpp:9-131) */
void compute_gradient(Oracle& o, State& Q) {
    const Mesh& m = o.m;
    const int nf = m.nf, nc = m.nc;
    Flow wall; wall.gamma = o.fs.gamma;
    vd sx[4], sy[4], fsx[4], fsy[4];
    for (int k = 0; k < 4; k++) { sx[k].assign(nc, 0); sy[k].assign(nc, 0); fsx[k].resize(nf); fsy[k].resize(nf); }
    const vd* Qp[4] = {&Q.p1, &Q.p2, &Q.p3, &Q.p4};
    for (int f = 0; f < nf; f++) {
        const int c1 = m.fc1[f], c2 = m.fc2[f];
        double d[4];
        switch (c2) {
            case -1:
                d[0] = o.fs.Q1 - Q.p1[c1]; d[1] = o.fs.Q2 - Q.p2[c1];
                d[2] = o.fs.Q3 - Q.p3[c1]; d[3] = o.fs.Q4 - Q.p4[c1];
                break;
            case -2: {
                wall.rho = Q.rho[c1];
                wall.P = Q.P[c1];
                double Vn = Q.u[c1] * m.nx[f] + Q.v[c1] * m.ny[f];
                wall.u = Q.u[c1] - 2.0 * Vn * m.nx[f];
                wall.v = Q.v[c1] - 2.0 * Vn * m.ny[f];
                wall.updateQ();
                d[0] = wall.Q1 - Q.p1[c1]; d[1] = wall.Q2 - Q.p2[c1];
                d[2] = wall.Q3 - Q.p3[c1]; d[3] = wall.Q4 - Q.p4[c1];
                break;
            }
            case -3:
                d[0] = 0; d[1] = 0; d[2] = 0; d[3] = 0;
                break;
            case -4:
                /* cell_gradient.cpp:63-66: the ghost reads cell number `face index` */
                wall.rho = Q.rho[f];
                wall.P = Q.P[f];
                wall.u = -Q.u[f];
                wall.v = -Q.v[f];
                wall.updateQ();
                d[0] = wall.Q1 - Q.p1[c1]; d[1] = wall.Q2 - Q.p2[c1];
                d[2] = wall.Q3 - Q.p3[c1]; d[3] = wall.Q4 - Q.p4[c1];
                break;
            default:
                for (int k = 0; k < 4; k++) d[k] = (*Qp[k])[c2] - (*Qp[k])[c1];
                break;
        }
        for (int k = 0; k < 4; k++) { fsx[k][f] = d[k] * m.dxj[f]; fsy[k][f] = d[k] * m.dyj[f]; }
    }
    for (int f = 0; f < nf; f++) {                     /* cell_gradient.cpp:93-118 */
        const int c1 = m.fc1[f], c2 = m.fc2[f];
        for (int k = 0; k < 4; k++) { sx[k][c1] += fsx[k][f]; sy[k][c1] += fsy[k][f]; }
        if (c2 >= 0) for (int k = 0; k < 4; k++) { sx[k][c2] += fsx[k][f]; sy[k][c2] += fsy[k][f]; }
    }
    vd* Qx[4] = {&Q.Qxp1, &Q.Qxp2, &Q.Qxp3, &Q.Qxp4};
    vd* Qy[4] = {&Q.Qyp1, &Q.Qyp2, &Q.Qyp3, &Q.Qyp4};
    for (int c = 0; c < nc; c++)                       /* cell_gradient.cpp:120-130 */
        for (int k = 0; k < 4; k++) {
            (*Qx[k])[c] = (sx[k][c] * m.Iyy[c] - sy[k][c] * m.Ixy[c]);
            (*Qy[k])[c] = (sy[k][c] * m.Ixx[c] - sx[k][c] * m.Ixy[c]);
        }
}

inline double min2(double a, double b) { return (b < a) ? b : a; }   /* std::min({a, b}) */
inline double max2(double a, double b) { return (a < b) ? b : a; }   /* std::max({a, b}) */

/* squeeze (src/solver/squeeze.cpp:9-155).  Qface_c1/c2 hold the face values of the previous
 * res() call (res.cpp:40 runs before the reconstruction at :48).                             */
void squeeze(Oracle& o, State& Q) {
    const Mesh& m = o.m;
    const int nf = m.nf, nc = m.nc;
    const vd* Qp[4] = {&Q.p1, &Q.p2, &Q.p3, &Q.p4};
    const vd* F1[4] = {&o.Qface_c1.p1, &o.Qface_c1.p2, &o.Qface_c1.p3, &o.Qface_c1.p4};
    const vd* F2[4] = {&o.Qface_c2.p1, &o.Qface_c2.p2, &o.Qface_c2.p3, &o.Qface_c2.p4};
    vd qmin[4], qmax[4];
    for (int k = 0; k < 4; k++) { qmin[k].assign(nc, 100000000000); qmax[k].assign(nc, -100000000000); }
    for (int f = 0; f < nf; f++) {                     /* squeeze.cpp:17-62 */
        const int c1 = m.fc1[f], c2 = m.fc2[f];
        for (int k = 0; k < 4; k++) {
            const vd& q = *Qp[k];
            double tmin, tmax;
            if (c2 >= 0) {
                tmin = min2(q[c1], q[c2]);
                tmax = max2(q[c1], q[c2]);
                qmin[k][c2] = min2(qmin[k][c2], tmin);
                qmax[k][c2] = max2(qmax[k][c2], tmax);
            } else {
                tmin = q[c1];
                tmax = q[c1];
            }
            qmin[k][c1] = min2(qmin[k][c1], tmin);
            qmax[k][c1] = max2(qmax[k][c1], tmax);
        }
    }
    vd ph1[4], ph2[4];
    for (int k = 0; k < 4; k++) { ph1[k].assign(nf, 1); ph2[k].assign(nf, 1); }
    for (int f = 0; f < nf; f++) {                     /* squeeze.cpp:68-121 */
        const int c1 = m.fc1[f], c2 = m.fc2[f];
        for (int k = 0; k < 4; k++) {
            const vd& q = *Qp[k];
            double qf = (*F1[k])[f];
            if (qf < qmin[k][c1]) ph1[k][f] = (qmin[k][c1] - q[c1]) / (qf - q[c1]);
            else if (qf > qmax[k][c1]) ph1[k][f] = (qmax[k][c1] - q[c1]) / (qf - q[c1]);
            if (c2 >= 0) {   /* the reference also evaluates BC faces (out of bounds); unused */
                qf = (*F2[k])[f];
                if (qf < qmin[k][c2]) ph2[k][f] = (qmin[k][c2] - q[c2]) / (qf - q[c2]);
                else if (qf > qmax[k][c2]) ph2[k][f] = (qmax[k][c2] - q[c2]) / (qf - q[c2]);
            }
        }
    }
    vd phi[4];
    for (int k = 0; k < 4; k++) phi[k].assign(nc, 1);
    static const int korder[4] = {0, 3, 1, 2};         /* squeeze.cpp:126-141 updates p1, p4, p2, p3 */
    for (int f = 0; f < nf; f++) {
        const int c1 = m.fc1[f], c2 = m.fc2[f];
        for (int kk = 0; kk < 4; kk++) { int k = korder[kk]; phi[k][c1] = min2(ph1[k][f], phi[k][c1]); }
        if (c2 >= 0) for (int kk = 0; kk < 4; kk++) { int k = korder[kk]; phi[k][c2] = min2(ph2[k][f], phi[k][c2]); }
    }
    vd* Qx[4] = {&Q.Qxp1, &Q.Qxp2, &Q.Qxp3, &Q.Qxp4};
    vd* Qy[4] = {&Q.Qyp1, &Q.Qyp2, &Q.Qyp3, &Q.Qyp4};
    for (int c = 0; c < nc; c++)                       /* squeeze.cpp:144-154 */
        for (int k = 0; k < 4; k++) {
            (*Qx[k])[c] = (*Qx[k])[c] * phi[k][c];
            (*Qy[k])[c] = (*Qy[k])[c] * phi[k][c];
        }
}

/* reconstruction (src/solver/reconstruction.cpp:15-168) */
void reconstruction(Oracle& o, State& Q) {
    const Mesh& m = o.m;
    const int nf = m.nf;
    State& L = o.Qface_c1;
    State& Rt = o.Qface_c2;
    Flow wall; wall.gamma = o.fs.gamma;
    for (int f = 0; f < nf; f++) {                     /* reconstruction.cpp:22-79 */
        const int c1 = m.fc1[f], c2 = m.fc2[f];
        L.p1[f] = Q.p1[c1] + Q.Qxp1[c1] * m.c1dx[f] + Q.Qyp1[c1] * m.c1dy[f];
        L.p2[f] = Q.p2[c1] + Q.Qxp2[c1] * m.c1dx[f] + Q.Qyp2[c1] * m.c1dy[f];
        L.p3[f] = Q.p3[c1] + Q.Qxp3[c1] * m.c1dx[f] + Q.Qyp3[c1] * m.c1dy[f];
        L.p4[f] = Q.p4[c1] + Q.Qxp4[c1] * m.c1dx[f] + Q.Qyp4[c1] * m.c1dy[f];
        L.updateflow_int(f);
        switch (c2) {
            case -1:
                Rt.p1[f] = o.fs.Q1; Rt.p2[f] = o.fs.Q2; Rt.p3[f] = o.fs.Q3; Rt.p4[f] = o.fs.Q4;
                break;
            case -2: {
                wall.rho = L.rho[f];
                wall.P = L.P[f];
                double Vn = L.u[f] * m.nx[f] + L.v[f] * m.ny[f];
                wall.u = L.u[f] - 2.0 * Vn * m.nx[f];
                wall.v = L.v[f] - 2.0 * Vn * m.ny[f];
                wall.updateQ();
                Rt.p1[f] = wall.Q1; Rt.p2[f] = wall.Q2; Rt.p3[f] = wall.Q3; Rt.p4[f] = wall.Q4;
                break;
            }
            case -3:
                Rt.p1[f] = L.p1[f]; Rt.p2[f] = L.p2[f]; Rt.p3[f] = L.p3[f]; Rt.p4[f] = L.p4[f];
                break;
            case -4:
                wall.rho = L.rho[f];
                wall.P = L.P[f];
                wall.u = -L.u[f];
                wall.v = -L.v[f];
                wall.updateQ();
                Rt.p1[f] = wall.Q1; Rt.p2[f] = wall.Q2; Rt.p3[f] = wall.Q3; Rt.p4[f] = wall.Q4;
                break;
            default:
                Rt.p1[f] = Q.p1[c2] + Q.Qxp1[c2] * m.c2dx[f] + Q.Qyp1[c2] * m.c2dy[f];
                Rt.p2[f] = Q.p2[c2] + Q.Qxp2[c2] * m.c2dx[f] + Q.Qyp2[c2] * m.c2dy[f];
                Rt.p3[f] = Q.p3[c2] + Q.Qxp3[c2] * m.c2dx[f] + Q.Qyp3[c2] * m.c2dy[f];
                Rt.p4[f] = Q.p4[c2] + Q.Qxp4[c2] * m.c2dx[f] + Q.Qyp4[c2] * m.c2dy[f];
                break;
        }
    }
    Rt.updateflow();
    if (o.cs.eqn != 2) return;
    State& A = o.Qface;                                /* reconstruction.cpp:86-92 */
    for (int f = 0; f < nf; f++) {
        A.p1[f] = 0.5 * (L.p1[f] + Rt.p1[f]);
        A.p2[f] = 0.5 * (L.p2[f] + Rt.p2[f]);
        A.p3[f] = 0.5 * (L.p3[f] + Rt.p3[f]);
        A.p4[f] = 0.5 * (L.p4[f] + Rt.p4[f]);
    }
    A.updateflow();
    const double gm1 = o.fs.gamma - 1;
    for (int f = 0; f < nf; f++) {                     /* reconstruction.cpp:96-164 */
        const int c1 = m.fc1[f], c2 = m.fc2[f];
        switch (c2) {
            case -1:
            case -3:
                A.comp_vis(f, 0, 0, 0, 0, 0, 0, 0, 0);
                break;
            case -2:
                /* reconstruction.cpp:104-106: prints an error and leaves tau / grad T as they were */
                break;
            case -4: {
                double dn = std::abs(std::sqrt(m.c1dx[f] * m.c1dx[f] + m.c1dy[f] * m.c1dy[f]));
                double dudn = -Q.u[c1] / dn;
                double dvdn = -Q.v[c1] / dn;
                double dudx = dudn * m.nx[f], dudy = dudn * m.ny[f];
                double dvdx = dvdn * m.nx[f], dvdy = dvdn * m.ny[f];
                A.comp_vis(f, dudx, dudy, dvdx, dvdy, 0, 0, 0, 0);
                break;
            }
            default: {
                const double ad = std::abs(m.dist[f]);
                const double l1 = (Q.p1[c2] - Q.p1[c1]) / ad;
                const double l2 = (Q.p2[c2] - Q.p2[c1]) / ad;
                const double l3 = (Q.p3[c2] - Q.p3[c1]) / ad;
                const double l4 = (Q.p4[c2] - Q.p4[c1]) / ad;
                const double mx = m.mx[f], my = m.my[f];
                const double m1 = 0.5 * (Q.Qxp1[c1] * mx + Q.Qyp1[c1] * my + Q.Qxp1[c2] * mx + Q.Qyp1[c2] * my);
                const double m2 = 0.5 * (Q.Qxp2[c1] * mx + Q.Qyp2[c1] * my + Q.Qxp2[c2] * mx + Q.Qyp2[c2] * my);
                const double m3 = 0.5 * (Q.Qxp3[c1] * mx + Q.Qyp3[c1] * my + Q.Qxp3[c2] * mx + Q.Qyp3[c2] * my);
                const double m4 = 0.5 * (Q.Qxp4[c1] * mx + Q.Qyp4[c1] * my + Q.Qxp4[c2] * mx + Q.Qyp4[c2] * my);
                const double lx = m.lx[f], ly = m.ly[f];
                const double y1 = l1 * ly + m1 * ly, y2 = l2 * ly + m2 * ly;
                const double y3 = l3 * ly + m3 * ly, y4 = l4 * ly + m4 * ly;
                const double x1 = l1 * lx + m1 * lx, x2 = l2 * lx + m2 * lx;
                const double x3 = l3 * lx + m3 * lx, x4 = l4 * lx + m4 * lx;
                const double ru = A.u[f], rv = A.v[f], rr = A.rho[f];
                const double drhodx = x1;
                const double dudx = x2 - drhodx * ru / rr;
                const double dvdx = x3 - drhodx * rv / rr;
                const double drhody = y1;
                const double dudy = y2 - drhody * ru / rr;
                const double dvdy = y3 - drhody * ru / rr;   /* reconstruction.cpp:155 uses u */
                const double dPdx = gm1 * (x4 - 0.5 * drhodx * (ru * ru + rv * rv) - rr * (ru * dudx + rv * dvdx));
                const double dPdy = gm1 * (y4 - 0.5 * drhody * (ru * ru + rv * rv) - rr * (ru * dudy + rv * dvdy));
                A.comp_vis(f, dudx, dudy, dvdx, dvdy, dPdx, dPdy, drhodx, drhody);
                break;
            }
        }
    }
}

/* res (src/solver/res.cpp:21-110) with class_F::update / update_vis (class_f.hpp:41-59) and
 * rusanov (src/solver/rusanov.cpp:12-37).                                                    */
void res(Oracle& o, State& Q) {
    const Mesh& m = o.m;
    const int nf = m.nf, nc = m.nc;
    vd Fp[4], Fv[4];
    for (int k = 0; k < 4; k++) { Fp[k].assign(nf, -101); Fv[k].assign(nf, 0); }
    if (o.cs.order == 1) {
        reconstruction(o, Q);
    } else if (o.cs.order == 2) {
        compute_gradient(o, Q);
        if (o.cs.limiter == 2) squeeze(o, Q);
        reconstruction(o, Q);
        if (o.cs.eqn == 2) {
            const State& A = o.Qface;
            for (int f = 0; f < nf; f++) {
                Fv[0][f] = 0;
                Fv[1][f] = A.tau_xx[f] * m.nx[f] + A.tau_xy[f] * m.ny[f];
                Fv[2][f] = A.tau_xy[f] * m.nx[f] + A.tau_yy[f] * m.ny[f];
                Fv[3][f] = m.nx[f] * (A.u[f] * A.tau_xx[f] + A.v[f] * A.tau_xy[f] + A.k * A.dTdx[f]) +
                           m.ny[f] * (A.u[f] * A.tau_xy[f] + A.v[f] * A.tau_yy[f] + A.k * A.dTdy[f]);
            }
        }
    }
    if (o.cs.flux_solver == 1) {
        State& L = o.Qface_c1;
        State& Rt = o.Qface_c2;
        for (int f = 0; f < nf; f++) {
            const double nx = m.nx[f], ny = m.ny[f];
            const double vn1 = L.u[f] * nx + L.v[f] * ny;
            const double vn2 = Rt.u[f] * nx + Rt.v[f] * ny;
            const double a1 = L.rho[f] * vn1, a2 = Rt.rho[f] * vn2;
            const double b1 = L.rho[f] * L.u[f] * vn1 + L.P[f] * nx, b2 = Rt.rho[f] * Rt.u[f] * vn2 + Rt.P[f] * nx;
            const double e1 = L.rho[f] * L.v[f] * vn1 + L.P[f] * ny, e2 = Rt.rho[f] * Rt.v[f] * vn2 + Rt.P[f] * ny;
            const double g1 = vn1 * (L.E[f] + L.P[f]), g2 = vn2 * (Rt.E[f] + Rt.P[f]);
            const double vna = (vn1 + vn2) / 2;
            const double ca = (L.c[f] + Rt.c[f]) / 2;
            L.Vn_avg[f] = vna; L.c_avg[f] = ca; Rt.Vn_avg[f] = vna; Rt.c_avg[f] = ca;
            Fp[0][f] = (a1 + a2) / 2 - (std::abs(vna) + ca) / 2 * (Rt.p1[f] - L.p1[f]);
            Fp[1][f] = (b1 + b2) / 2 - (std::abs(vna) + ca) / 2 * (Rt.p2[f] - L.p2[f]);
            Fp[2][f] = (e1 + e2) / 2 - (std::abs(vna) + ca) / 2 * (Rt.p3[f] - L.p3[f]);
            Fp[3][f] = (g1 + g2) / 2 - (std::abs(vna) + ca) / 2 * (Rt.p4[f] - L.p4[f]);
        }
    }
    vd* r[4] = {&o.r1, &o.r2, &o.r3, &o.r4};
    for (int k = 0; k < 4; k++) std::fill(r[k]->begin(), r[k]->end(), 0.0);
    for (int f = 0; f < nf; f++) {                     /* res.cpp:74-102 */
        const int c1 = m.fc1[f], c2 = m.fc2[f];
        for (int k = 0; k < 4; k++) {
            const double s = (Fp[k][f] * m.area[f]);
            const double sv = (Fv[k][f] * m.area[f]);
            (*r[k])[c1] += sv - s;
            if (c2 >= 0) (*r[k])[c2] -= sv - s;
        }
    }
    for (int c = 0; c < nc; c++)                       /* res.cpp:104-109 */
        for (int k = 0; k < 4; k++) (*r[k])[c] = (*r[k])[c] / m.vol[c];
}

/* time step (src/solver/ssp_rk3.cpp:24-47), from the Vn_avg / c_avg of the previous res() */
void compute_dt(Oracle& o) {
    const Mesh& m = o.m;
    std::fill(o.dt.begin(), o.dt.end(), 0.0);
    for (int f = 0; f < m.nf; f++) {
        const int c1 = m.fc1[f], c2 = m.fc2[f];
        o.dt[c1] += (std::abs(o.Qface_c1.Vn_avg[f]) + o.Qface_c1.c_avg[f]) * m.area[f];
        if (c2 >= 0) o.dt[c2] += (std::abs(o.Qface_c2.Vn_avg[f]) + o.Qface_c2.c_avg[f]) * m.area[f];
    }
    if (o.cs.type == 1) {
        double mx = *std::max_element(o.dt.begin(), o.dt.end());
        for (int c = 0; c < m.nc; c++) o.dt[c] = (2 * o.cs.CFL * m.vol[c]) / mx;
    } else if (o.cs.type == 2) {
        for (int c = 0; c < m.nc; c++) o.dt[c] = (2 * o.cs.CFL * m.vol[c]) / o.dt[c];
    }
}

/* one SSP-RK3 stage (src/solver/ssp_rk3.cpp:50-77); three calls make one ssp_rk3() */
void do_stage(Oracle& o) {
    const int N = o.m.nc;
    State& Qs = o.Qstar;
    const vd* rr[4] = {&o.r1, &o.r2, &o.r3, &o.r4};
    vd* qb[4] = {&o.Qbar.p1, &o.Qbar.p2, &o.Qbar.p3, &o.Qbar.p4};
    vd* qs[4] = {&Qs.p1, &Qs.p2, &Qs.p3, &Qs.p4};
    if (o.stage == 0) {
        Qs.init(N, o.fs.gamma, o.fs.R);                /* ssp_rk3.cpp:20-21 */
        o.have_qstar = true;
        compute_dt(o);
        res(o, o.Qbar);
        for (int c = 0; c < N; c++)
            for (int k = 0; k < 4; k++) (*qs[k])[c] = (*qb[k])[c] + o.dt[c] * (*rr[k])[c];
        Qs.updateflow();
    } else if (o.stage == 1) {
        res(o, Qs);
        for (int c = 0; c < N; c++)
            for (int k = 0; k < 4; k++)
                (*qs[k])[c] = 0.75 * (*qb[k])[c] + 0.25 * (*qs[k])[c] + 0.25 * o.dt[c] * (*rr[k])[c];
        Qs.updateflow();
    } else {
        res(o, Qs);
        for (int c = 0; c < N; c++)
            for (int k = 0; k < 4; k++)
                (*qb[k])[c] = (1.0 / 3.0) * (*qb[k])[c] + (2.0 / 3.0) * (*qs[k])[c] + (2.0 / 3.0) * o.dt[c] * (*rr[k])[c];
        o.Qbar.updateflow();
    }
    o.stage = (o.stage + 1) % 3;
}

int copy_out(const vd& a, double* out, int off) {
    std::copy(a.begin(), a.end(), out + off);
    return off + (int)a.size();
}

Oracle* finish_open(Oracle* o, const vi& fp1, const vi& fp2, const vi& fc1, const vi& fc2) {
    if (o->cs.order != 1 && o->cs.order != 2) { delete o; return nullptr; }
    /* RUSANOV (1) or ROE (2): with ROE the reference's res() calls no flux routine (res.cpp:62-69), so
     * the inviscid flux keeps class_F::init's -101 (class_f.hpp:26-30) and Vn_avg / c_avg keep their
     * initial values (class_q.hpp:61-62); res() above reproduces both by skipping the Rusanov block */
    if (o->cs.flux_solver != 1 && o->cs.flux_solver != 2) { delete o; return nullptr; }
    for (int f = 0; f < o->m.nf; f++) {
        if (fc1[f] < 1 || fc1[f] > o->m.nc || fc2[f] < -1 || fc2[f] > o->m.nc ||
            fp1[f] < 1 || fp1[f] > o->m.np || fp2[f] < 1 || fp2[f] > o->m.np) { delete o; return nullptr; }
    }
    build_connectivity(o->m, o->cs, fp1.data(), fp2.data(), fc1.data(), fc2.data());
    /* a NO_SLIP_WALL face reads cell number `face id` in the gradient (cell_gradient.cpp:63) */
    for (int f = 0; f < o->m.nf; f++)
        if (o->m.fc2[f] == -4 && f >= o->m.nc) { delete o; return nullptr; }
    build_geometry(o->m);
    setup(*o);
    return o;
}

}  // namespace

extern "C" {

void* fvo_open(const char* input_file) {
    Oracle* o = new Oracle();
    if (!read_inputs(input_file, o->cs, o->fs)) { delete o; return nullptr; }
    /* like the reference, a relative grid path is relative to the working directory */
    vi fp1, fp2, fc1, fc2;
    if (!read_grid_file(o->cs.grid_file.c_str(), o->m, fp1, fp2, fc1, fc2)) { delete o; return nullptr; }
    return finish_open(o, fp1, fp2, fc1, fc2);
}

void* fvo_open_arrays(const fvo_case* c, int np, int nf, int nc, const double* x, const double* y,
                      const int* fp1, const int* fp2, const int* fc1, const int* fc2) {
    Oracle* o = new Oracle();
    o->cs.order = c->order; o->cs.eqn = c->eqn; o->cs.flux_solver = c->flux_solver;
    o->cs.limiter = c->limiter; o->cs.type = c->time_type; o->cs.scheme = c->time_scheme;
    o->cs.BC1 = c->bc1; o->cs.BC2 = c->bc2; o->cs.CFL = c->cfl;
    o->fs.gamma = c->gamma; o->fs.R = c->R; o->fs.mu = c->mu; o->fs.Pr = c->Pr;
    o->fs.P = c->P; o->fs.rho = c->rho; o->fs.u = c->u; o->fs.v = c->v;
    o->m.np = np; o->m.nf = nf; o->m.nc = nc;
    o->m.x.assign(x, x + np); o->m.y.assign(y, y + np);
    vi a(fp1, fp1 + nf), b(fp2, fp2 + nf), c1(fc1, fc1 + nf), c2(fc2, fc2 + nf);
    return finish_open(o, a, b, c1, c2);
}

void fvo_close(void* h) { delete (Oracle*)h; }

void fvo_sizes(void* h, int* out) {
    Oracle* o = (Oracle*)h;
    out[0] = o->m.np; out[1] = o->m.nf; out[2] = o->m.nc; out[3] = o->m.numBC1;
    out[4] = o->m.numBC2; out[5] = o->m.numWALL; out[6] = o->m.num_of_BC; out[7] = o->stage;
}

void fvo_stage(void* h) { do_stage(*(Oracle*)h); }

void fvo_iterate(void* h, int n) {
    for (int i = 0; i < 3 * n; i++) do_stage(*(Oracle*)h);
}

double fvo_time_iterations(void* h, int n) {
    auto t0 = std::chrono::steady_clock::now();
    fvo_iterate(h, n);
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

void fvo_set_state(void* h, const double* q) {
    /* restart path (main.cpp:82-106, 114-118): fresh face states, Qbar.init(N, gamma, R),
     * read p1..p4, updateflow */
    Oracle* o = (Oracle*)h;
    const int N = o->m.nc, F = o->m.nf;
    if (o->cs.eqn == 2) o->Qface.init(F, o->fs);
    o->Qface_c1.init(F, o->fs);
    o->Qface_c2.init(F, o->fs);
    o->Qbar.init(N, o->fs.gamma, o->fs.R);
    for (int c = 0; c < N; c++) {
        o->Qbar.p1[c] = q[c]; o->Qbar.p2[c] = q[N + c]; o->Qbar.p3[c] = q[2 * N + c]; o->Qbar.p4[c] = q[3 * N + c];
    }
    o->Qbar.updateflow();
    o->stage = 0;
}

int fvo_get(void* h, int field, double* out) {
    Oracle* o = (Oracle*)h;
    const Mesh& m = o->m;
    int n = 0;
    switch (field) {
        case FVO_QBAR: n = copy_out(o->Qbar.p1, out, 0); n = copy_out(o->Qbar.p2, out, n);
                       n = copy_out(o->Qbar.p3, out, n); n = copy_out(o->Qbar.p4, out, n); break;
        case FVO_QSTAR: if (!o->have_qstar) return -1;
                       n = copy_out(o->Qstar.p1, out, 0); n = copy_out(o->Qstar.p2, out, n);
                       n = copy_out(o->Qstar.p3, out, n); n = copy_out(o->Qstar.p4, out, n); break;
        case FVO_RES: n = copy_out(o->r1, out, 0); n = copy_out(o->r2, out, n);
                      n = copy_out(o->r3, out, n); n = copy_out(o->r4, out, n); break;
        case FVO_DT: n = copy_out(o->dt, out, 0); break;
        case FVO_QBAR_GRAD: case FVO_QSTAR_GRAD: {
            if (field == FVO_QSTAR_GRAD && !o->have_qstar) return -1;
            const State& s = (field == FVO_QBAR_GRAD) ? o->Qbar : o->Qstar;
            for (const vd* a : {&s.Qxp1, &s.Qxp2, &s.Qxp3, &s.Qxp4, &s.Qyp1, &s.Qyp2, &s.Qyp3, &s.Qyp4})
                n = copy_out(*a, out, n);
            break;
        }
        case FVO_QF1: n = copy_out(o->Qface_c1.p1, out, 0); n = copy_out(o->Qface_c1.p2, out, n);
                      n = copy_out(o->Qface_c1.p3, out, n); n = copy_out(o->Qface_c1.p4, out, n); break;
        case FVO_QF2: n = copy_out(o->Qface_c2.p1, out, 0); n = copy_out(o->Qface_c2.p2, out, n);
                      n = copy_out(o->Qface_c2.p3, out, n); n = copy_out(o->Qface_c2.p4, out, n); break;
        case FVO_VNC: n = copy_out(o->Qface_c1.Vn_avg, out, 0); n = copy_out(o->Qface_c1.c_avg, out, n); break;
        case FVO_QBAR_PRIM: n = copy_out(o->Qbar.rho, out, 0); n = copy_out(o->Qbar.u, out, n);
                            n = copy_out(o->Qbar.v, out, n); n = copy_out(o->Qbar.P, out, n); break;
        case FVO_G_AREA: n = copy_out(m.area, out, 0); break;
        case FVO_G_NX: n = copy_out(m.nx, out, 0); break;
        case FVO_G_NY: n = copy_out(m.ny, out, 0); break;
        case FVO_G_FCX: n = copy_out(m.fcx, out, 0); break;
        case FVO_G_FCY: n = copy_out(m.fcy, out, 0); break;
        case FVO_G_C1DX: n = copy_out(m.c1dx, out, 0); break;
        case FVO_G_C1DY: n = copy_out(m.c1dy, out, 0); break;
        case FVO_G_C2DX: n = copy_out(m.c2dx, out, 0); break;
        case FVO_G_C2DY: n = copy_out(m.c2dy, out, 0); break;
        case FVO_G_DXJ: n = copy_out(m.dxj, out, 0); break;
        case FVO_G_DYJ: n = copy_out(m.dyj, out, 0); break;
        case FVO_G_DIST: n = copy_out(m.dist, out, 0); break;
        case FVO_G_LX: n = copy_out(m.lx, out, 0); break;
        case FVO_G_LY: n = copy_out(m.ly, out, 0); break;
        case FVO_G_MX: n = copy_out(m.mx, out, 0); break;
        case FVO_G_MY: n = copy_out(m.my, out, 0); break;
        case FVO_G_VOL: n = copy_out(m.vol, out, 0); break;
        case FVO_G_CCX: n = copy_out(m.ccx, out, 0); break;
        case FVO_G_CCY: n = copy_out(m.ccy, out, 0); break;
        case FVO_G_IXX: n = copy_out(m.Ixx, out, 0); break;
        case FVO_G_IYY: n = copy_out(m.Iyy, out, 0); break;
        case FVO_G_IXY: n = copy_out(m.Ixy, out, 0); break;
        case FVO_G_DELTA: n = copy_out(m.delta, out, 0); break;
        case FVO_G_BCCX: n = copy_out(m.bccx, out, 0); break;
        case FVO_G_BCCY: n = copy_out(m.bccy, out, 0); break;
        default: return -1;
    }
    return n;
}

int fvo_get_int(void* h, int field, int* out) {
    Oracle* o = (Oracle*)h;
    const Mesh& m = o->m;
    const vi* a = nullptr;
    switch (field) {
        case FVO_I_FC1: a = &m.fc1; break;
        case FVO_I_FC2: a = &m.fc2; break;
        case FVO_I_FP1: a = &m.fp1; break;
        case FVO_I_FP2: a = &m.fp2; break;
        case FVO_I_CFC: a = &m.cf_count; break;
        case FVO_I_BCF: a = &m.BC_faces; break;
        default: return -1;
    }
    std::copy(a->begin(), a->end(), out);
    return (int)a->size();
}

}  // extern "C"
