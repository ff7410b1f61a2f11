// Solution output in the reference's file layout: monitor line + sol/output.dat +
// sol/res_history.dat (save_sol.cpp:17-103), node-averaged Tecplot volume and surface files
// (save_sol.cpp:105-234), the restart file (post_process.cpp:13-29) and readmesh's mesh dumps
// (readmesh.cpp:413-446).  Values are written with the default C++ stream formatting (6
// significant digits) and computed with the reference's expressions, so for bit-identical inputs
// the files are byte-identical.  Compile with -ffp-contract=off.
#include "fv2d_output.h"

#include <cmath>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

namespace fv2d {

namespace {
// unique vertices of a cell in discovery order, as readmesh.cpp:147-185 finds them
void cell_vertices(const HostMesh& m, int c, std::vector<double>& vx, std::vector<double>& vy) {
    const int b = m.cf_off[c], e = m.cf_off[c + 1], n = e - b;
    vx.assign(n, 0.0);
    vy.assign(n, 0.0);
    int found = 0;
    auto add = [&](double px, double py) {
        for (int z = 0; z < n; z++) if (vx[z] == px && vy[z] == py) return;
        if (found < n) { vx[found] = px; vy[found] = py; found++; }
    };
    for (int k = b; k < e; k++) {
        const int f = m.cf[k];
        add(m.x[m.fp1[f]], m.y[m.fp1[f]]);
        add(m.x[m.fp2[f]], m.y[m.fp2[f]]);
    }
}
}  // namespace

int write_mesh_files(const HostMesh& m, const std::string& dir, std::string& err) {
    std::ofstream out(dir + "/cell_data.dat");
    if (!out.is_open()) { err = "cannot write " + dir + "/cell_data.dat"; return FV2D_ERR_IO; }
    out << "# cell_vol, cell_centerx, cell_centery, x points for cell, y points for cell" << std::endl;
    std::vector<double> vx, vy;
    for (int c = 0; c < m.nc; c++) {
        cell_vertices(m, c, vx, vy);
        double sx[6], sy[6];   // six vertex slots, unused ones -101 (readmesh.cpp:144-145)
        for (int j = 0; j < 6; j++) { sx[j] = j < (int)vx.size() ? vx[j] : -101; sy[j] = j < (int)vy.size() ? vy[j] : -101; }
        out << m.vol[c] << " " << m.ccx[c] << " " << m.ccy[c] << " ";
        out << sx[0] << " " << sx[1] << " " << sx[2] << " " << sx[3] << " " << sx[4] << " " << sx[5] << " ";
        out << sy[0] << " " << sy[1] << " " << sy[2] << " " << sy[3] << " " << sy[4] << " " << sy[5] << std::endl;
    }
    out.close();
    out.open(dir + "/face_data.dat");
    if (!out.is_open()) { err = "cannot write " + dir + "/face_data.dat"; return FV2D_ERR_IO; }
    out << "# face point 1 x, face point 1 y, face point 2 x, face point 2y, face nx, face ny, face center x, face center y" << std::endl;
    for (int f = 0; f < m.nf; f++) {
        out << m.x[m.fp1[f]] << " " << m.y[m.fp1[f]] << " ";
        out << m.x[m.fp2[f]] << " " << m.y[m.fp2[f]] << " ";
        out << m.nx[f] << " " << m.ny[f] << " ";
        out << m.fcx[f] << " " << m.fcy[f] << std::endl;
    }
    return FV2D_OK;
}

int write_history_headers(const std::string& dir, std::string& err) {
    std::ofstream a(dir + "/res_history.dat");
    if (!a.is_open()) { err = "cannot write " + dir + "/res_history.dat"; return FV2D_ERR_IO; }
    a << "#iter, res1, res2, res3, res4" << std::endl;
    std::ofstream b(dir + "/output.dat");
    if (!b.is_open()) { err = "cannot write " + dir + "/output.dat"; return FV2D_ERR_IO; }
    b << "#iter, CL, CD" << std::endl;
    return FV2D_OK;
}

// q, r: SoA 4N; g: 8N (Qx p1..p4, Qy p1..p4), all in the reference's numbering.
int save_solution(const HostMesh& m, const fv2d_case& cs, int ndx, const double* q, const double* g, const double* r,
                  const std::string& dir, std::string& err) {
    const int N = m.nc, NP = m.np;
    const double gamma = cs.gamma, mu = cs.mu;
    const double* Q[4] = {q, q + N, q + 2 * (size_t)N, q + 3 * (size_t)N};
    const double* QX[4] = {g, g + N, g + 2 * (size_t)N, g + 3 * (size_t)N};
    const double* QY[4] = {g + 4 * (size_t)N, g + 5 * (size_t)N, g + 6 * (size_t)N, g + 7 * (size_t)N};
    const double* R[4] = {r, r + N, r + 2 * (size_t)N, r + 3 * (size_t)N};
    const int numWALL = m.numWALL < 0 ? 0 : m.numWALL;
    auto cell_u = [&](int c) { return Q[1][c] / Q[0][c]; };   // Qbar->u after updateflow (class_q.hpp:131-141)
    auto cell_v = [&](int c) { return Q[2][c] / Q[0][c]; };
    if (cs.monitor_step > 0 && (ndx % cs.monitor_step) == 0) {                 // save_sol.cpp:18-103
        double Fy = 0, Fx = 0;
        for (int idx = 0; idx < numWALL; idx++) {
            const int face = idx;                      // wall faces are taken to be faces 0..numWALL-1
            const int c1 = m.fc1[face];
            const int cellx = (int)m.ccx[c1], celly = (int)m.ccy[c1];   // truncated, as save_sol.cpp:28-32
            const int facex = (int)m.fcx[face], facey = (int)m.fcy[face];
            double fr[4];
            for (int k = 0; k < 4; k++) fr[k] = Q[k][c1] + ((facex - cellx) * QX[k][c1] + (facey - celly) * QY[k][c1]);
            const double rho = fr[0], u = fr[1] / rho, v = fr[2] / rho, E = fr[3];
            const double P = (E - (0.5 * rho * (u * u + v * v))) * (gamma - 1);
            if (cs.eqn == FV2D_NS) {
                const double dn = std::abs(std::sqrt(m.c1dx[face] * m.c1dx[face] + m.c1dy[face] * m.c1dy[face]));
                const double dudn = -cell_u(c1) / dn, dvdn = -cell_v(c1) / dn;
                const double tx = mu * dudn, ty = mu * dvdn;
                const double tw = std::sqrt(tx * tx + ty * ty);
                if (m.ny[face] < 0) {
                    Fx += tw * m.area[face] * (-m.ny[face]);
                    Fy += tw * m.area[face] * (m.nx[face]);
                } else {
                    Fx += tw * m.area[face] * (m.ny[face]);
                    Fy += tw * m.area[face] * (-m.nx[face]);
                }
            }
            const double force = P * m.area[face];
            Fy += force * m.ny[face];
            Fx += force * m.nx[face];
        }
        const double norm = std::sqrt(cs.u * cs.u + cs.v * cs.v);       // class_flow::free_comp
        const double flowx = cs.u / norm, flowy = cs.v / norm;
        const double L = Fx * (-flowy) + Fy * flowx;
        const double D = Fy * flowy + Fx * flowx;
        const double Vmag = std::sqrt(cs.u * cs.u + cs.v * cs.v);
        const double CL = L / (0.5 * cs.rho * Vmag * Vmag * cs.length);
        const double CD = D / (0.5 * cs.rho * Vmag * Vmag * cs.length);
        double res[4] = {0, 0, 0, 0};
        for (int c = 0; c < N; c++)
            for (int k = 0; k < 4; k++) res[k] += R[k][c] * R[k][c];
        for (int k = 0; k < 4; k++) res[k] = std::sqrt(res[k]);
        std::cout << "iter: " << ndx << ", CL: " << CL << ", CD: " << CD << ", res: " << res[0] << ", " << res[1]
                  << ", " << res[2] << ", " << res[3] << std::endl;
        std::ofstream output(dir + "/output.dat", std::ios_base::app | std::ios_base::out);
        output << ndx << " " << CL << " " << CD << std::endl;
        std::ofstream hist(dir + "/res_history.dat", std::ios_base::app | std::ios_base::out);
        hist << ndx << " " << res[0] << " " << res[1] << " " << res[2] << " " << res[3] << std::endl;
        if (!output || !hist) { err = "cannot append to " + dir + "/output.dat or res_history.dat"; return FV2D_ERR_IO; }
    }
    if (cs.output_step > 0 && (ndx % cs.output_step) == 0) {                   // save_sol.cpp:106-234
        std::cout << "Saving Solution \n";
        std::vector<int> cnt(NP, 0);
        std::vector<double> pa[4];
        for (int k = 0; k < 4; k++) pa[k].assign(NP, 0.0);
        for (int f = 0; f < m.nf; f++) {
            const int c1 = m.fc1[f], c2 = m.fc2[f], p1 = m.fp1[f], p2 = m.fp2[f];
            cnt[p1]++;
            cnt[p2]++;
            for (int k = 0; k < 4; k++)
                pa[k][p1] += Q[k][c1] + ((m.x[p1] - m.ccx[c1]) * QX[k][c1] + (m.y[p1] - m.ccy[c1]) * QY[k][c1]);
            for (int k = 0; k < 4; k++)
                pa[k][p2] += Q[k][c1] + ((m.x[p2] - m.ccx[c1]) * QX[k][c1] + (m.y[p2] - m.ccy[c1]) * QY[k][c1]);
            if (c2 >= 0) {
                for (int k = 0; k < 4; k++)
                    pa[k][p1] += Q[k][c2] + ((m.x[p1] - m.ccx[c2]) * QX[k][c2] + (m.y[p1] - m.ccy[c2]) * QY[k][c2]);
                for (int k = 0; k < 4; k++)
                    pa[k][p2] += Q[k][c2] + ((m.x[p2] - m.ccx[c2]) * QX[k][c2] + (m.y[p2] - m.ccy[c2]) * QY[k][c2]);
                cnt[p1]++;
                cnt[p2]++;
            }
        }
        for (int p = 0; p < NP; p++)
            for (int k = 0; k < 4; k++) pa[k][p] = pa[k][p] / (cnt[p]);
        std::vector<double> prho(NP), pE(NP), pu(NP), pv(NP), pP(NP);
        for (int p = 0; p < NP; p++) {
            prho[p] = pa[0][p];
            pE[p] = pa[3][p];
            pu[p] = pa[1][p] / prho[p];
            pv[p] = pa[2][p] / prho[p];
            pP[p] = (pE[p] - (0.5 * prho[p] * (pu[p] * pu[p] + pv[p] * pv[p]))) * (gamma - 1);
        }
        std::vector<double> tau_x(numWALL + 1, 0.0), tau_y(numWALL + 1, 0.0);   // entry numWALL: see below
        if (cs.eqn == FV2D_NS) {
            for (int idx = 0; idx < numWALL; idx++) {
                const int face = m.bc_faces[idx], c1 = m.fc1[face];
                const double dn = std::abs(std::sqrt(m.c1dx[face] * m.c1dx[face] + m.c1dy[face] * m.c1dy[face]));
                tau_x[idx] = mu * (-cell_u(c1) / dn);
                tau_y[idx] = mu * (-cell_v(c1) / dn);
            }
        }
        const bool last = cs.nmax == ndx;
        std::ofstream out(dir + (last ? std::string("/tec_sol.dat") : "/tec_sol_" + std::to_string(ndx) + ".dat"));
        if (!out.is_open()) { err = "cannot write the Tecplot volume file"; return FV2D_ERR_IO; }
        out << "VARIABLES = \"X\", \"Y\", \"density\", \"u\", \"v\", \"P\" \n";
        out << "Zone STRANDID=1, ZoneType=FETRIANGLE, SOLUTIONTIME=" << ndx << std::endl;
        out << "n=" << m.nf << " e=" << m.nf * 2 - m.num_of_BC << " DATAPACKING=POINT" << std::endl;   // n= prints faces
        out << "DT=(DOUBLE DOUBLE DOUBLE DOUBLE DOUBLE DOUBLE )" << std::endl;
        for (int p = 0; p < NP; p++) {
            out << m.x[p] << " " << m.y[p] << " ";
            out << prho[p] << " " << pu[p] << " " << pv[p] << " " << pP[p] << std::endl;
        }
        for (int c = 0; c < N; c++) {
            const double rho = Q[0][c], u = cell_u(c), v = cell_v(c);
            const double P = (Q[3][c] - (0.5 * rho * (u * u + v * v))) * (gamma - 1);
            out << m.ccx[c] << " " << m.ccy[c] << " ";
            out << rho << " " << u << " " << v << " " << P << std::endl;
        }
        for (int c = 0; c < N; c++)                                          // readmesh.cpp:342-353
            for (int k = m.cf_off[c]; k < m.cf_off[c + 1]; k++) {
                const int f = m.cf[k];
                out << (double)(m.fp1[f] + 1) << " " << (double)(m.fp2[f] + 1) << " " << (double)(NP + c + 1) << std::endl;
            }
        out.close();
        out.open(dir + (last ? std::string("/tec_surf.dat") : "/tec_surf_" + std::to_string(ndx) + ".dat"));
        if (!out.is_open()) { err = "cannot write the Tecplot surface file"; return FV2D_ERR_IO; }
        out << "TITLE     = \"Translation of CGNS file merged_sol_aver.cgns\"" << std::endl;
        out << "VARIABLES = \"CoordinateX\" \n \"CoordinateY\" \n \"rho\" \n \"u\" \n \"v\" \n \"P\" \n \"tau_x\" \n \"tau_y\" " << std::endl;
        out << "ZONE T=\"ZONE1\"\nSTRANDID=0, SOLUTIONTIME=" << ndx << "\nI=" << numWALL + 1 << ", J=1, K=1, ZONETYPE=Ordered\n";
        out << "DATAPACKING=POINT\nDT=(DOUBLE DOUBLE DOUBLE DOUBLE DOUBLE DOUBLE )\n";
        // numWALL + 1 rows (save_sol.cpp:227): the reference reads tau one past its end on the last
        // row; here that entry is 0
        for (int idx = 0; idx < numWALL + 1 && idx < NP; idx++) {
            out << m.x[idx] << " " << m.y[idx] << " ";
            out << prho[idx] << " " << pu[idx] << " " << pv[idx] << " " << pP[idx] << " " << tau_x[idx] << " " << tau_y[idx] << std::endl;
        }
    }
    return FV2D_OK;
}

int write_restart_file(const HostMesh& m, const std::string& path, int ndx, const double* q, int digits,
                       std::string& err) {
    std::ofstream out(path);
    if (!out.is_open()) { err = "cannot write " + path; return FV2D_ERR_IO; }
    if (digits > 0) out.precision(digits);   // 17 round-trips every double exactly
    const int N = m.nc;
    out << ndx << " " << N << std::endl;
    for (int c = 0; c < N; c++)
        out << q[c] << " " << q[N + c] << " " << q[2 * (size_t)N + c] << " " << q[3 * (size_t)N + c] << std::endl;
    if (!out) { err = "write failed: " + path; return FV2D_ERR_IO; }
    return FV2D_OK;
}

int write_restart(const HostMesh& m, int ndx, const double* q, const std::string& dir, std::string& err) {
    std::cout << "Writing Restart File \n";                                   // post_process.cpp:13-29
    return write_restart_file(m, dir + "/restart_sol.dat", ndx, q, 0, err);   // stream default: 6 digits
}

int read_restart(const char* path, int num_cells, int* ndx, double* q, std::string& err) {
    std::ifstream in(path);                                                     // main.cpp:83-104
    if (!in.is_open()) { err = std::string("cannot open restart file ") + path; return FV2D_ERR_IO; }
    int n = 0;
    in >> *ndx >> n;
    if (!in || n != num_cells) { err = "restart file does not match the grid (cell count)"; return FV2D_ERR_IO; }
    for (int c = 0; c < n; c++) {
        double a, b, cc, d;
        in >> a >> b >> cc >> d;
        q[c] = a; q[n + c] = b; q[2 * (size_t)n + c] = cc; q[3 * (size_t)n + c] = d;
    }
    if (!in) { err = "restart file truncated"; return FV2D_ERR_IO; }
    return FV2D_OK;
}

}  // namespace fv2d
