// Host mesh build for the GB300 fv2d library.  Compile with -ffp-contract=off: the geometry must
// round exactly like the reference's (src/base/readmesh.cpp) on x86-64 and on aarch64 hosts.
#include "fv2d_host.h"

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <numeric>
#include <sstream>

namespace fv2d {

// ------------------------------------------------------------------------------------ input.in
// Same token rules as read_inputs (src/base/read_inputs.cpp:17-209): nine section tokens, each
// followed by a fixed number of `key = value` triples; unknown string values leave the field as
// it was.  Fields the file never sets stay 0 here (the reference leaves them uninitialised).
int parse_inputs(const char* path, fv2d_case* cs, std::string& err) {
    std::memset(cs, 0, sizeof(*cs));
    std::ifstream in(path);
    if (!in.is_open()) { err = std::string("cannot open input file ") + path; return FV2D_ERR_IO; }
    std::string key, eq, val;
    auto next = [&]() -> bool { return (bool)(in >> key >> eq >> val); };
    const struct { const char* name; int count; } sections[] = {
        {"[case]", 5}, {"[limiter]", 1}, {"[grid]", 1}, {"[equations]", 2}, {"[fluid]", 4},
        {"[init]", 4}, {"[time]", 3}, {"[report]", 1}, {"[BC]", 2}};
    auto bc_code = [](const std::string& s, int& dst) {
        if (s == "FREESTREAM") dst = FV2D_BC_FREESTREAM;
        if (s == "SLIP_WALL") dst = FV2D_BC_SLIP_WALL;
        if (s == "EXTRAPOLATION") dst = FV2D_BC_EXTRAPOLATION;
        if (s == "NO_SLIP_WALL") dst = FV2D_BC_NO_SLIP_WALL;
    };
    try {
        for (int s = 0; s < 9; s++) {
            std::string tok;
            if (!(in >> tok)) break;
            int count = 0;
            for (const auto& sec : sections) if (tok == sec.name) count = sec.count;
            for (int j = 0; j < count; j++) {
                if (!next()) break;
                if (tok == "[case]") {
                    if (key == "solution_poly_order") cs->order = std::stoi(val) + 1;
                    if (key == "nmax") cs->nmax = std::stoi(val);
                    if (key == "monitor_step") cs->monitor_step = std::stoi(val);
                    if (key == "output_step") cs->output_step = std::stoi(val);
                    if (key == "restart") cs->restart = std::stoi(val);
                } else if (tok == "[limiter]") {
                    if (key == "limiter") {
                        if (val == "NONE") cs->limiter = FV2D_LIM_NONE;
                        if (val == "MINMOD") cs->limiter = FV2D_LIM_MINMOD;
                        if (val == "SQUEEZE") cs->limiter = FV2D_LIM_SQUEEZE;
                    }
                } else if (tok == "[grid]") {
                    if (key == "grid_file") std::snprintf(cs->grid_file, sizeof(cs->grid_file), "%s", val.c_str());
                } else if (tok == "[equations]") {
                    if (key == "eqn") { if (val == "EULER") cs->eqn = FV2D_EULER; if (val == "NS") cs->eqn = FV2D_NS; }
                    if (key == "flux_solver") { if (val == "RUSANOV") cs->flux_solver = FV2D_RUSANOV; if (val == "ROE") cs->flux_solver = FV2D_ROE; }
                } else if (tok == "[fluid]") {
                    if (key == "gamma") cs->gamma = std::stod(val);
                    if (key == "R") cs->R = std::stod(val);
                    if (key == "mu") cs->mu = std::stod(val);
                    if (key == "Pr") cs->Pr = std::stod(val);
                } else if (tok == "[init]") {
                    if (key == "P") cs->P = std::stod(val);
                    if (key == "rho") cs->rho = std::stod(val);
                    if (key == "u") cs->u = std::stod(val);
                    if (key == "v") cs->v = std::stod(val);
                } else if (tok == "[time]") {
                    if (key == "CFL") cs->cfl = std::stod(val);
                    if (key == "time_step_type") { if (val == "GLOBAL") cs->time_type = FV2D_DT_GLOBAL; if (val == "LOCAL") cs->time_type = FV2D_DT_LOCAL; }
                    if (key == "time_scheme") { if (val == "SSP_RK2") cs->time_scheme = FV2D_SSP_RK2; if (val == "SSP_RK3") cs->time_scheme = FV2D_SSP_RK3; }
                } else if (tok == "[report]") {
                    if (key == "length") cs->length = std::stod(val);
                } else if (tok == "[BC]") {
                    if (key == "BC1") bc_code(val, cs->bc1);
                    if (key == "BC2") bc_code(val, cs->bc2);
                }
            }
        }
    } catch (const std::exception& e) {
        err = std::string("malformed value in ") + path + ": '" + val + "' for key '" + key + "'";
        return FV2D_ERR_IO;
    }
    return FV2D_OK;
}

// ------------------------------------------------------------------------------------ grid file
namespace {
struct Cursor {
    const char* p;
    const char* end;
    bool ok = true;
    void skip() { while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t' || *p == '\f' || *p == '\v')) p++; }
    long geti() {
        skip();
        if (p >= end) { ok = false; return 0; }
        char* e;
        errno = 0;
        long v = std::strtol(p, &e, 10);
        if (e == p || errno) { ok = false; return 0; }
        p = e;
        return v;
    }
    double getd() {
        skip();
        if (p >= end) { ok = false; return 0; }
        char* e;
        double v = std::strtod(p, &e);   // correctly rounded, as istream >> double
        if (e == p) { ok = false; return 0; }
        p = e;
        return v;
    }
};
}  // namespace

int parse_grid(const char* path, std::vector<double>& x, std::vector<double>& y, std::vector<int>& fp1,
               std::vector<int>& fp2, std::vector<int>& fc1, std::vector<int>& fc2, int& nc, std::string& err) {
    FILE* fh = std::fopen(path, "rb");
    if (!fh) { err = std::string("cannot open grid file ") + path; return FV2D_ERR_IO; }
    std::fseek(fh, 0, SEEK_END);
    long len = std::ftell(fh);
    std::fseek(fh, 0, SEEK_SET);
    std::string buf;
    buf.resize(len > 0 ? (size_t)len + 1 : 1);
    size_t got = len > 0 ? std::fread(&buf[0], 1, (size_t)len, fh) : 0;
    std::fclose(fh);
    buf[got] = '\0';
    Cursor c{buf.data(), buf.data() + got};
    long np = c.geti(), nf = c.geti(), ncl = c.geti();
    if (!c.ok || np <= 0 || nf <= 0 || ncl <= 0 || np > INT32_MAX / 2 || nf > INT32_MAX / 4 || ncl > INT32_MAX / 2) {
        err = std::string("bad grid header in ") + path;
        return FV2D_ERR_IO;
    }
    x.resize(np); y.resize(np);
    for (long i = 0; i < np; i++) { x[i] = c.getd(); y[i] = c.getd(); }
    fp1.resize(nf); fp2.resize(nf); fc1.resize(nf); fc2.resize(nf);
    for (long f = 0; f < nf; f++) { fp1[f] = (int)c.geti(); fp2[f] = (int)c.geti(); }
    for (long f = 0; f < nf; f++) { fc1[f] = (int)c.geti(); fc2[f] = (int)c.geti(); }
    if (!c.ok) { err = std::string("grid file truncated or malformed: ") + path; return FV2D_ERR_IO; }
    nc = (int)ncl;
    return FV2D_OK;
}

int write_grid(const char* path, const fv2d_mesh_desc* d, std::string& err) {
    FILE* fh = std::fopen(path, "wb");
    if (!fh) { err = std::string("cannot write grid file ") + path; return FV2D_ERR_IO; }
    std::vector<char> buf(size_t(1) << 22);
    size_t used = 0;
    bool ok = true;
    auto flush = [&]() {
        if (used && std::fwrite(buf.data(), 1, used, fh) != used) ok = false;
        used = 0;
    };
    auto room = [&](size_t n) { if (used + n > buf.size()) flush(); };
    room(64);
    used += (size_t)std::snprintf(buf.data() + used, 64, "%d %d %d\n", d->num_points, d->num_faces, d->num_cells);
    for (int i = 0; i < d->num_points; i++) {   // 17 significant digits: every double round-trips
        room(64);
        used += (size_t)std::snprintf(buf.data() + used, 64, "%.17g %.17g\n", d->x[i], d->y[i]);
    }
    for (int f = 0; f < d->num_faces; f++) {
        room(32);
        used += (size_t)std::snprintf(buf.data() + used, 32, "%d %d\n", d->face_point1[f], d->face_point2[f]);
    }
    for (int f = 0; f < d->num_faces; f++) {
        room(32);
        used += (size_t)std::snprintf(buf.data() + used, 32, "%d %d\n", d->face_cell1[f], d->face_cell2[f]);
    }
    flush();
    if (std::fclose(fh) != 0) ok = false;
    if (!ok) { err = std::string("write failed: ") + path; return FV2D_ERR_IO; }
    return FV2D_OK;
}

// ------------------------------------------------------------------------------------ mesh build
namespace {

// Connectivity and BC tagging (readmesh.cpp:50-85, 356-360).
int connectivity(const fv2d_mesh_desc* d, const fv2d_case* cs, HostMesh& m, std::string& err) {
    const int nf = m.nf, nc = m.nc, np = m.np;
    m.fp1.resize(nf); m.fp2.resize(nf); m.fc1.resize(nf); m.fc2.resize(nf);
    m.face2bc.assign(nf, -1);
    m.bc_faces.clear();
    std::vector<int> cnt(nc, 0);
    m.numBC1 = m.numBC2 = 0;
    for (int f = 0; f < nf; f++) {
        const int p1 = d->face_point1[f], p2 = d->face_point2[f];
        const int c1 = d->face_cell1[f], c2 = d->face_cell2[f];
        if (p1 < 1 || p1 > np || p2 < 1 || p2 > np || p1 == p2) {
            err = "face " + std::to_string(f + 1) + ": point id out of range or degenerate"; return FV2D_ERR_MESH;
        }
        if (c1 < 1 || c1 > nc || c2 < -1 || c2 > nc || c1 == c2) {
            err = "face " + std::to_string(f + 1) + ": cell id out of range (c2 must be a cell, 0 or -1)"; return FV2D_ERR_MESH;
        }
        m.fp1[f] = p1 - 1;
        m.fp2[f] = p2 - 1;
        m.fc1[f] = c1 - 1;
        if (c2 == 0) { m.fc2[f] = cs->bc1; m.numBC1++; }
        else if (c2 == -1) { m.fc2[f] = cs->bc2; m.numBC2++; }
        else m.fc2[f] = c2 - 1;
        cnt[c1 - 1]++;
        if (c2 > 0) cnt[c2 - 1]++;
        if (c2 <= 0) { m.face2bc[f] = (int)m.bc_faces.size(); m.bc_faces.push_back(f); }
    }
    m.num_of_BC = (int)m.bc_faces.size();
    m.cf_off.assign(nc + 1, 0);
    m.max_sides = 0;
    for (int c = 0; c < nc; c++) {
        if (cnt[c] < 3) { err = "cell " + std::to_string(c + 1) + " has fewer than 3 faces"; return FV2D_ERR_MESH; }
        m.cf_off[c + 1] = m.cf_off[c] + cnt[c];
        m.max_sides = std::max(m.max_sides, cnt[c]);
    }
    m.cf.assign(m.cf_off[nc], -1);
    std::vector<int> fill(m.cf_off.begin(), m.cf_off.end() - 1);
    for (int f = 0; f < nf; f++) {
        m.cf[fill[m.fc1[f]]++] = f;
        if (m.fc2[f] >= 0) m.cf[fill[m.fc2[f]]++] = f;
    }
    m.numWALL = -1;   // left unset by the reference when neither BC is a wall
    if (cs->bc1 == FV2D_BC_SLIP_WALL || cs->bc1 == FV2D_BC_NO_SLIP_WALL) m.numWALL = m.numBC1;
    else if (cs->bc2 == FV2D_BC_SLIP_WALL || cs->bc2 == FV2D_BC_NO_SLIP_WALL) m.numWALL = m.numBC2;
    return FV2D_OK;
}

// Geometry (readmesh.cpp:117-411), same expressions and summation order.
void geometry(HostMesh& m) {
    const int nf = m.nf, nc = m.nc;
    m.area.resize(nf); m.nx.resize(nf); m.ny.resize(nf); m.fcx.resize(nf); m.fcy.resize(nf);
    m.mx.resize(nf); m.my.resize(nf);
    for (int f = 0; f < nf; f++) {
        const double xa = m.x[m.fp1[f]], ya = m.y[m.fp1[f]];
        const double dx = m.x[m.fp2[f]] - xa, dy = m.y[m.fp2[f]] - ya;
        const double a = sqrt(dx * dx + dy * dy);
        m.area[f] = a;
        m.nx[f] = dy / a;
        m.ny[f] = -dx / a;
        m.fcx[f] = dx / 2 + xa;
        m.fcy[f] = dy / 2 + ya;
        // unit tangent p1 -> p2 (readmesh.cpp:400-406)
        const double t = std::sqrt(dx * dx + dy * dy);
        m.mx[f] = dx / t;
        m.my[f] = dy / t;
    }
    // cells: vertex mean as the fan centre, fan-triangle areas, area-weighted centroid
    m.vol.resize(nc); m.ccx.resize(nc); m.ccy.resize(nc);
    std::vector<double> vx(m.max_sides), vy(m.max_sides);
    for (int c = 0; c < nc; c++) {
        const int b = m.cf_off[c], e = m.cf_off[c + 1], n = e - b;
        // unique vertices in discovery order; unfilled slots read as (0, 0) like the reference's
        // zero-initialised scratch (readmesh.cpp:149-185)
        std::fill(vx.begin(), vx.begin() + n, 0.0);
        std::fill(vy.begin(), vy.begin() + n, 0.0);
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
        double sx = 0, sy = 0;
        for (int z = 0; z < n; z++) { sx += vx[z]; sy += vy[z]; }
        const double cx = sx / n, cy = sy / n;
        double sv = 0, scx = 0, scy = 0;
        for (int k = b; k < e; k++) {
            const int f = m.cf[k];
            const double x1 = m.x[m.fp1[f]], y1 = m.y[m.fp1[f]];
            const double x2 = m.x[m.fp2[f]], y2 = m.y[m.fp2[f]];
            const double tri = 0.5 * std::abs(x1 * (y2 - cy) + x2 * (cy - y1) + cx * (y1 - y2));
            sv += tri;
            scx += ((x1 + x2 + cx) / 3) * tri;
            scy += ((y1 + y2 + cy) / 3) * tri;
        }
        m.vol[c] = sv;
        m.ccx[c] = scx / sv;
        m.ccy[c] = scy / sv;
    }
    // ghost centres: mirror of the c1 centroid across the boundary face (readmesh.cpp:235-244)
    m.bccx.resize(m.num_of_BC); m.bccy.resize(m.num_of_BC);
    for (int i = 0; i < m.num_of_BC; i++) {
        const int f = m.bc_faces[i], c1 = m.fc1[f];
        const double rx = m.fcx[f] - m.ccx[c1], ry = m.fcy[f] - m.ccy[c1];
        const double s = 2.0 * (rx * m.nx[f] + ry * m.ny[f]);
        m.bccx[i] = m.ccx[c1] + s * m.nx[f];
        m.bccy[i] = m.ccy[c1] + s * m.ny[f];
    }
    // face-centre offsets, LSQ vectors and moments (readmesh.cpp:252-320)
    m.c1dx.resize(nf); m.c1dy.resize(nf); m.c2dx.resize(nf); m.c2dy.resize(nf);
    m.dxj.resize(nf); m.dyj.resize(nf);
    std::vector<double> sxx(nc, 0), syy(nc, 0), sxy(nc, 0);
    for (int f = 0; f < nf; f++) {
        const int c1 = m.fc1[f], c2 = m.fc2[f];
        const double xi = m.ccx[c1], yi = m.ccy[c1];
        const double xj = c2 >= 0 ? m.ccx[c2] : m.bccx[m.face2bc[f]];
        const double yj = c2 >= 0 ? m.ccy[c2] : m.bccy[m.face2bc[f]];
        m.c1dx[f] = m.fcx[f] - xi;
        m.c1dy[f] = m.fcy[f] - yi;
        m.c2dx[f] = m.fcx[f] - xj;
        m.c2dy[f] = m.fcy[f] - yj;
        sxx[c1] += (xi - xj) * (xi - xj);
        syy[c1] += (yi - yj) * (yi - yj);
        sxy[c1] += ((xi - xj) * (yi - yj));
        if (c2 >= 0) {
            sxx[c2] += (xj - xi) * (xj - xi);
            syy[c2] += (yj - yi) * (yj - yi);
            sxy[c2] += ((xj - xi) * (yj - yi));
        }
        m.dxj[f] = xj - xi;
        m.dyj[f] = yj - yi;
    }
    m.delta.resize(nc); m.Ixx.resize(nc); m.Iyy.resize(nc); m.Ixy.resize(nc);
    for (int c = 0; c < nc; c++) {
        const double dl = sxx[c] * syy[c] - (sxy[c] * sxy[c]);
        m.delta[c] = dl;
        m.Ixx[c] = sxx[c] / dl;
        m.Iyy[c] = syy[c] / dl;
        m.Ixy[c] = sxy[c] / dl;
    }
    // NS face frame (readmesh.cpp:363-411).  On boundary faces the reference looks the ghost up
    // through BC_faces[face id] (readmesh.cpp:373,394), which is only the right ghost when the
    // boundary faces come first; the NS terms never read these values on boundary faces, and
    // lookups outside the arrays give NaN here.
    const double qnan = std::numeric_limits<double>::quiet_NaN();
    m.dist.resize(nf); m.lx.resize(nf); m.ly.resize(nf);
    for (int f = 0; f < nf; f++) {
        const int c1 = m.fc1[f], c2 = m.fc2[f];
        double tx = qnan, ty = qnan;
        if (c2 >= 0) { tx = m.ccx[c2] - m.ccx[c1]; ty = m.ccy[c2] - m.ccy[c1]; }
        else if (f < m.num_of_BC && m.bc_faces[f] < m.num_of_BC) {
            const int g = m.bc_faces[f];
            tx = m.bccx[g] - m.ccx[c1]; ty = m.bccy[g] - m.ccy[c1];
        }
        m.dist[f] = std::sqrt(tx * tx + ty * ty);
        const double t2 = std::sqrt(tx * tx + ty * ty);
        m.lx[f] = tx / t2;
        m.ly[f] = ty / t2;
    }
}

void renumber(HostMesh& m) {
    const int nc = m.nc, nf = m.nf;
    double x0 = m.ccx[0], x1 = m.ccx[0], y0 = m.ccy[0], y1 = m.ccy[0];
    for (int c = 0; c < nc; c++) {
        x0 = std::min(x0, m.ccx[c]); x1 = std::max(x1, m.ccx[c]);
        y0 = std::min(y0, m.ccy[c]); y1 = std::max(y1, m.ccy[c]);
    }
    const double span = std::max(x1 - x0, y1 - y0);
    const double sc = span > 0 ? 65535.0 / span : 0.0;
    std::vector<uint64_t> key(nc);
    for (int c = 0; c < nc; c++) {
        double qx = (m.ccx[c] - x0) * sc, qy = (m.ccy[c] - y0) * sc;
        uint32_t ix = (uint32_t)std::min(65535.0, std::max(0.0, std::isfinite(qx) ? qx : 0.0));
        uint32_t iy = (uint32_t)std::min(65535.0, std::max(0.0, std::isfinite(qy) ? qy : 0.0));
        uint64_t d = 0;   // Hilbert index of (ix, iy) on a 65536^2 grid (xy -> d, quadrant by quadrant)
        for (uint32_t s = 1u << 15; s > 0; s >>= 1) {
            const uint32_t rx = (ix & s) ? 1u : 0u, ry = (iy & s) ? 1u : 0u;
            d += (uint64_t)s * s * ((3u * rx) ^ ry);
            if (ry == 0) {   // rotate the quadrant (the bits above s are not read again)
                if (rx == 1) { ix = 65535u - ix; iy = 65535u - iy; }
                std::swap(ix, iy);
            }
        }
        key[c] = (d << 32) | (uint32_t)c;
    }
    std::sort(key.begin(), key.end());
    // Within each run of kSideBlock Hilbert-consecutive cells (a small spatial patch), cells are
    // ordered by face count (stable): a warp's cells then loop over the same number of faces, so
    // the per-cell gathers do not wait for the warp's one many-sided cell.  Results do not depend
    // on the order (every per-cell sum runs in ascending original face id).
    constexpr int kSideBlock = 256;
    for (int b0 = 0; b0 < nc; b0 += kSideBlock) {
        const int b1 = std::min(nc, b0 + kSideBlock);
        std::stable_sort(key.begin() + b0, key.begin() + b1, [&](uint64_t a, uint64_t b) {
            const int ca = (int)(a & 0xFFFFFFFFu), cb = (int)(b & 0xFFFFFFFFu);
            return m.cf_off[ca + 1] - m.cf_off[ca] < m.cf_off[cb + 1] - m.cf_off[cb];
        });
    }
    m.cell_new2old.resize(nc);
    m.cell_old2new.resize(nc);
    for (int i = 0; i < nc; i++) {
        const int c = (int)(key[i] & 0xFFFFFFFFu);
        m.cell_new2old[i] = c;
        m.cell_old2new[c] = i;
    }
    // faces follow their first cell in the new order (ties by original id); boundary faces go after
    // all interior faces, so the face kernel's warps do not mix the boundary and interior branches
    std::vector<uint64_t> fk(nf);
    for (int f = 0; f < nf; f++)
        fk[f] = ((uint64_t)(m.fc2[f] < 0 ? 1 : 0) << 63) | ((uint64_t)m.cell_old2new[m.fc1[f]] << 32) | (uint32_t)f;
    std::sort(fk.begin(), fk.end());
    m.face_new2old.resize(nf);
    m.face_old2new.resize(nf);
    for (int i = 0; i < nf; i++) {
        const int f = (int)(fk[i] & 0xFFFFFFFFu);
        m.face_new2old[i] = f;
        m.face_old2new[f] = i;
    }
}

}  // namespace

int build_mesh(const fv2d_mesh_desc* d, const fv2d_case* cs, HostMesh& m, std::string& err) {
    if (!d || !cs || !d->x || !d->y || !d->face_point1 || !d->face_point2 || !d->face_cell1 || !d->face_cell2) {
        err = "null mesh array"; return FV2D_ERR_ARG;
    }
    if (d->num_points <= 0 || d->num_faces <= 0 || d->num_cells <= 0) { err = "empty mesh"; return FV2D_ERR_MESH; }
    m.np = d->num_points; m.nf = d->num_faces; m.nc = d->num_cells;
    m.bc1 = cs->bc1; m.bc2 = cs->bc2;
    m.x.assign(d->x, d->x + m.np);
    m.y.assign(d->y, d->y + m.np);
    int rc = connectivity(d, cs, m, err);
    if (rc) return rc;
    // The NO_SLIP_WALL gradient ghost reads cell number `face id` (src/solver/cell_gradient.cpp:63-66);
    // that cell only exists when the face id is below the cell count.
    for (int f = 0; f < m.nf; f++)
        if (m.fc2[f] == FV2D_BC_NO_SLIP_WALL && f >= m.nc) {
            err = "NO_SLIP_WALL face " + std::to_string(f + 1) +
                  " has an id >= num_cells: the reference gradient would read past its cell arrays; "
                  "write boundary faces first";
            return FV2D_ERR_MESH;
        }
    geometry(m);
    renumber(m);
    return FV2D_OK;
}

void build_layout(const HostMesh& m, DeviceLayout& L) {
    const int nc = m.nc, nf = m.nf;
    L.nc = nc; L.nf = nf;
    L.inc_off.assign(nc + 1, 0);
    for (int i = 0; i < nc; i++) {
        const int o = m.cell_new2old[i];
        L.inc_off[i + 1] = L.inc_off[i] + (m.cf_off[o + 1] - m.cf_off[o]);
    }
    L.ninc = L.inc_off[nc];
    L.inc.resize(L.ninc); L.nbr.resize(L.ninc); L.igeo.resize(4 * (size_t)L.ninc);
    for (int i = 0; i < nc; i++) {
        const int o = m.cell_new2old[i];
        int w = L.inc_off[i];
        for (int k = m.cf_off[o]; k < m.cf_off[o + 1]; k++, w++) {   // ascending original face id
            const int f = m.cf[k];
            const int side = (m.fc1[f] == o) ? 0 : 1;
            L.inc[w] = (m.face_old2new[f] << 1) | side;
            L.igeo[4 * (size_t)w + 0] = m.dxj[f];
            L.igeo[4 * (size_t)w + 1] = m.dyj[f];
            L.igeo[4 * (size_t)w + 2] = side == 0 ? m.c1dx[f] : m.c2dx[f];
            L.igeo[4 * (size_t)w + 3] = side == 0 ? m.c1dy[f] : m.c2dy[f];
            if (side == 0) L.nbr[w] = m.fc2[f] >= 0 ? m.cell_old2new[m.fc2[f]] : m.fc2[f];
            else L.nbr[w] = m.cell_old2new[m.fc1[f]];
        }
    }
    L.fc1.resize(nf); L.fc2.resize(nf); L.qcell.resize(nf);
    for (int g = 0; g < 14; g++) L.fgeo[g].resize(nf);
    const std::vector<double>* src[14] = {&m.nx, &m.ny, &m.area, &m.c1dx, &m.c1dy, &m.c2dx, &m.c2dy,
                                          &m.dxj, &m.dyj, &m.mx, &m.my, &m.lx, &m.ly, &m.dist};
    for (int i = 0; i < nf; i++) {
        const int f = m.face_new2old[i];
        L.fc1[i] = m.cell_old2new[m.fc1[f]];
        L.fc2[i] = m.fc2[f] >= 0 ? m.cell_old2new[m.fc2[f]] : m.fc2[f];
        L.qcell[i] = (m.fc2[f] == FV2D_BC_NO_SLIP_WALL) ? m.cell_old2new[f] : -1;
        for (int g = 0; g < 14; g++) L.fgeo[g][i] = (*src[g])[f];
    }
    L.vol.resize(nc); L.Ixx.resize(nc); L.Iyy.resize(nc); L.Ixy.resize(nc);
    for (int i = 0; i < nc; i++) {
        const int o = m.cell_new2old[i];
        L.vol[i] = m.vol[o]; L.Ixx[i] = m.Ixx[o]; L.Iyy[i] = m.Iyy[o]; L.Ixy[i] = m.Ixy[o];
    }
}

int mesh_field(const HostMesh& m, int field, double* out) {
    const std::vector<double>* a = nullptr;
    switch (field) {
        case FV2D_G_AREA: a = &m.area; break;
        case FV2D_G_NX: a = &m.nx; break;
        case FV2D_G_NY: a = &m.ny; break;
        case FV2D_G_FCX: a = &m.fcx; break;
        case FV2D_G_FCY: a = &m.fcy; break;
        case FV2D_G_C1DX: a = &m.c1dx; break;
        case FV2D_G_C1DY: a = &m.c1dy; break;
        case FV2D_G_C2DX: a = &m.c2dx; break;
        case FV2D_G_C2DY: a = &m.c2dy; break;
        case FV2D_G_DXJ: a = &m.dxj; break;
        case FV2D_G_DYJ: a = &m.dyj; break;
        case FV2D_G_DIST: a = &m.dist; break;
        case FV2D_G_LX: a = &m.lx; break;
        case FV2D_G_LY: a = &m.ly; break;
        case FV2D_G_MX: a = &m.mx; break;
        case FV2D_G_MY: a = &m.my; break;
        case FV2D_G_VOL: a = &m.vol; break;
        case FV2D_G_CCX: a = &m.ccx; break;
        case FV2D_G_CCY: a = &m.ccy; break;
        case FV2D_G_IXX: a = &m.Ixx; break;
        case FV2D_G_IYY: a = &m.Iyy; break;
        case FV2D_G_IXY: a = &m.Ixy; break;
        case FV2D_G_DELTA: a = &m.delta; break;
        case FV2D_G_BCCX: a = &m.bccx; break;
        case FV2D_G_BCCY: a = &m.bccy; break;
        default: return -1;
    }
    std::copy(a->begin(), a->end(), out);
    return (int)a->size();
}

}  // namespace fv2d
