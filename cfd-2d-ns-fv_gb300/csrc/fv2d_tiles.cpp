// Tile layout builder of the FP32 engine (see fv2d_tiles.h for the format).
#include "fv2d_tiles.h"

#include <algorithm>
#include <cstring>
#include <string>

#include "fv2d_host.h"

namespace fv2d {

namespace {

inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

inline uint32_t fbits(double v) {
    const float f = (float)v;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

// Scratch shared by the tiles of one mesh: per cell and per face, the tile that last marked it
// (stamps, so nothing is cleared between tiles) and its local slot / record index there.
struct Marks {
    std::vector<int> cstamp, cslot, fstamp, frec;
    explicit Marks(int nc, int nf) : cstamp(nc, -1), cslot(nc, 0), fstamp(nf, -1), frec(nf, 0) {}
};

// One tile's contents before it is appended.
struct Tile {
    int c0 = 0, ncore = 0;
    std::vector<int> ring1, ring2, faces;   // faces: new face ids in record order
    int ncc = 0, nint = 0, nrc = 0, ngeo = 0;
    std::vector<uint16_t> off;               // csr offsets (ngrad + 1)
    std::vector<uint32_t> ent;               // csr entries
};

// Gather the tile [c0, c0 + n): returns false when it exceeds a capacity.
bool make_tile(const DeviceLayout& L, int c0, int n, int stamp, Marks& mk, Tile& t) {
    t = Tile();
    t.c0 = c0;
    t.ncore = n;
    for (int i = 0; i < n; i++) { mk.cstamp[c0 + i] = stamp; mk.cslot[c0 + i] = i; }
    auto add_face = [&](int f) {
        if (mk.fstamp[f] == stamp) return;
        mk.fstamp[f] = stamp;
        t.faces.push_back(f);
    };
    // every face of a core cell (fluxes): faces between two core cells first (their fluxes need
    // only core gradients, so they can be evaluated while the ring-1 gradients are computed), then
    // the other interior faces, then boundary faces (warps do not mix the boundary branches);
    // new face id order within each group
    for (int c = c0; c < c0 + n; c++)
        for (int i = L.inc_off[c]; i < L.inc_off[c + 1]; i++) add_face(L.inc[i] >> 1);
    auto group = [&](int f) {
        const int a = L.fc1[f], b = L.fc2[f];
        if (b < 0) return 2;
        return (a >= c0 && a < c0 + n && b >= c0 && b < c0 + n) ? 0 : 1;
    };
    std::sort(t.faces.begin(), t.faces.end(), [&](int x, int y) {
        const int gx = group(x), gy = group(y);
        return gx != gy ? gx < gy : x < y;
    });
    t.ncc = 0;
    while (t.ncc < (int)t.faces.size() && group(t.faces[t.ncc]) == 0) t.ncc++;
    t.nint = t.ncc;
    while (t.nint < (int)t.faces.size() && group(t.faces[t.nint]) == 1) t.nint++;
    t.nrc = (int)t.faces.size();
    // ring 1: the other cells of those faces
    for (int k = 0; k < t.nrc; k++) {
        const int f = t.faces[k];
        for (int c : {L.fc1[f], L.fc2[f]})
            if (c >= 0 && mk.cstamp[c] != stamp) { mk.cstamp[c] = stamp; t.ring1.push_back(c); }
    }
    // by face count, then id: the ring-1 gradient pass runs one cell per thread, so a warp's cells
    // then loop over the same number of faces
    auto nfaces = [&](int c) { return L.inc_off[c + 1] - L.inc_off[c]; };
    std::sort(t.ring1.begin(), t.ring1.end(), [&](int x, int y) {
        const int fx = nfaces(x), fy = nfaces(y);
        return fx != fy ? fx < fy : x < y;
    });
    for (size_t k = 0; k < t.ring1.size(); k++) mk.cslot[t.ring1[k]] = n + (int)k;
    // the other faces of ring-1 cells (their gradients): boundary faces first (they carry the
    // normal, which the slip-wall ghost needs), then interior faces
    std::vector<int> bc, in;
    for (int c : t.ring1)
        for (int i = L.inc_off[c]; i < L.inc_off[c + 1]; i++) {
            const int f = L.inc[i] >> 1;
            if (mk.fstamp[f] == stamp) continue;
            mk.fstamp[f] = stamp;
            (L.fc2[f] < 0 ? bc : in).push_back(f);
        }
    std::sort(bc.begin(), bc.end());
    std::sort(in.begin(), in.end());
    t.faces.insert(t.faces.end(), bc.begin(), bc.end());
    t.ngeo = (int)t.faces.size();
    t.faces.insert(t.faces.end(), in.begin(), in.end());
    // ring 2: the other cells of the gradient-only faces
    for (int f : in)
        for (int c : {L.fc1[f], L.fc2[f]})
            if (c >= 0 && mk.cstamp[c] != stamp) { mk.cstamp[c] = stamp; t.ring2.push_back(c); }
    std::sort(t.ring2.begin(), t.ring2.end());
    const int n1 = (int)t.ring1.size(), n2 = (int)t.ring2.size();
    for (int k = 0; k < n2; k++) mk.cslot[t.ring2[k]] = n + n1 + k;
    const int nr = (int)t.faces.size();
    if (n + n1 > kTileGrad || n + n1 + n2 > kTileCells || nr > kTileRecs || t.ngeo > kTileGeo) return false;
    for (int k = 0; k < nr; k++) mk.frec[t.faces[k]] = k;
    // csr of the gradient cells (core, then ring 1), each in ascending original face id
    const int ngrad = n + n1;
    t.off.assign(ngrad + 1, 0);
    auto emit = [&](int c, int g) {
        bool bcf = false;
        for (int i = L.inc_off[c]; i < L.inc_off[c + 1]; i++) {
            const int f = L.inc[i] >> 1, side = L.inc[i] & 1;
            const int other = side ? mk.cslot[L.fc1[f]] : (L.fc2[f] >= 0 ? mk.cslot[L.fc2[f]] : L.fc2[f]);
            bcf = bcf || other < 0;
            t.ent.push_back((uint32_t)((mk.frec[f] << 1) | side) | ((uint32_t)(other & 0xFFFF) << 16));
        }
        // bit 15 of a cell's end offset: the cell has a boundary face
        t.off[g + 1] = (uint16_t)(t.ent.size() | (bcf ? 0x8000u : 0u));
    };
    for (int i = 0; i < n; i++) emit(c0 + i, i);
    for (int k = 0; k < n1; k++) emit(t.ring1[k], n + k);
    return round_up(ngrad + 1, 8) + 2 * round_up((int)t.ent.size(), 4) <= kTileCsr;
}

void append_tile(const HostMesh& m, const DeviceLayout& L, const Tile& t, Marks& mk, TileLayout& T) {
    (void)m;
    TileRec r;
    r.c0 = t.c0; r.ncore = t.ncore; r.n1 = (int)t.ring1.size(); r.n2 = (int)t.ring2.size();
    r.ncc = t.ncc; r.nint = t.nint; r.nrc = t.nrc; r.ngeo = t.ngeo; r.nr = (int)t.faces.size();
    r.nrp = round_up(r.nr, 4); r.ngp = round_up(r.ngeo, 4);
    r.noff = round_up((int)t.off.size(), 8);
    r.ncsr = r.noff + 2 * round_up((int)t.ent.size(), 4);
    r.nhalo = round_up(r.n1 + r.n2, 4);
    r.rec = (long long)T.rec.size();
    r.rbase = (long long)T.qcell.size();
    r.csr = (long long)T.csr.size();
    r.halo = (long long)T.halo.size();
    // record block
    T.rec.resize(T.rec.size() + 5 * (size_t)r.nrp + 3 * (size_t)r.ngp, 0u);
    uint32_t* b = T.rec.data() + r.rec;
    auto slot = [&](int c) { return mk.cslot[c]; };
    for (int k = 0; k < r.nr; k++) {
        const int f = t.faces[k];
        const int s1 = slot(L.fc1[f]);
        const int s2 = L.fc2[f] >= 0 ? slot(L.fc2[f]) : L.fc2[f];
        b[k] = (uint32_t)(s1 & 0xFFFF) | ((uint32_t)(s2 & 0xFFFF) << 16);
        uint32_t* d = b + r.nrp + 4 * (size_t)k;   // one 16-byte row per record
        d[0] = fbits(L.fgeo[3][f]);   // c1dx
        d[1] = fbits(L.fgeo[4][f]);   // c1dy
        d[2] = fbits(L.fgeo[5][f]);   // c2dx
        d[3] = fbits(L.fgeo[6][f]);   // c2dy
        if (k < r.ngeo) {
            b[5 * r.nrp + k] = fbits(L.fgeo[0][f]);                 // nx
            b[5 * r.nrp + r.ngp + k] = fbits(L.fgeo[1][f]);         // ny
            b[5 * r.nrp + 2 * r.ngp + k] = fbits(L.fgeo[2][f]);     // area
        }
        T.qcell.push_back(L.qcell[f]);
    }
    // csr block
    T.csr.resize(T.csr.size() + r.ncsr, (uint16_t)0);
    std::copy(t.off.begin(), t.off.end(), T.csr.begin() + r.csr);
    for (size_t e = 0; e < t.ent.size(); e++) {   // little-endian halves, as the device reads them
        T.csr[r.csr + r.noff + 2 * e] = (uint16_t)(t.ent[e] & 0xFFFFu);
        T.csr[r.csr + r.noff + 2 * e + 1] = (uint16_t)(t.ent[e] >> 16);
    }
    // halo list
    T.halo.insert(T.halo.end(), t.ring1.begin(), t.ring1.end());
    T.halo.insert(T.halo.end(), t.ring2.begin(), t.ring2.end());
    T.halo.resize(r.halo + r.nhalo, 0);
    T.tiles.push_back(r);
}

}  // namespace

bool check_tile_layout(const TileLayout& T, const DeviceLayout& L, std::string& err) {
    auto fail = [&](size_t t, const char* what) {
        err = "tile " + std::to_string(t) + ": " + what;
        return false;
    };
    long long cells = 0;
    for (size_t t = 0; t < T.tiles.size(); t++) {
        const TileRec& r = T.tiles[t];
        const int ncell = r.ncore + r.n1 + r.n2, ngrad = r.ncore + r.n1;
        if (r.ncore < 1 || r.ncore > kTileCore || ngrad > kTileGrad || ncell > kTileCells) return fail(t, "cell counts");
        if (r.c0 != cells) return fail(t, "core cells not contiguous");
        cells += r.ncore;
        if (r.ncc < 0 || r.ncc > r.nint || r.nint > r.nrc || r.nrc > r.ngeo || r.ngeo > r.nr || r.nr > kTileRecs || r.ngeo > kTileGeo)
            return fail(t, "record counts");
        if (r.nrp < r.nr || r.ngp < r.ngeo || (r.nrp & 3) || (r.ngp & 3) || 5 * r.nrp + 3 * r.ngp > 5 * kTileRecs + 3 * kTileGeo)
            return fail(t, "record block shape");
        if ((r.rec & 3) || (r.csr & 7) || (r.halo & 3) || (r.ncsr & 7) || (r.noff & 7) || (r.nhalo & 3) || r.ncsr > kTileCsr ||
            r.noff < ngrad + 1 || r.noff > r.ncsr || r.nhalo < r.n1 + r.n2 || r.nhalo > kTileCells)
            return fail(t, "block alignment or size");
        if (r.rec + 5 * (long long)r.nrp + 3 * (long long)r.ngp > (long long)T.rec.size() ||
            r.csr + r.ncsr > (long long)T.csr.size() || r.halo + r.nhalo > (long long)T.halo.size() ||
            r.rbase + r.nr > (long long)T.qcell.size())
            return fail(t, "block outside its array");
        for (int h = 0; h < r.n1 + r.n2; h++) {
            const int c = T.halo[r.halo + h];
            if (c < 0 || c >= T.nc || (c >= r.c0 && c < r.c0 + r.ncore)) return fail(t, "halo id");
        }
        const uint32_t* b = T.rec.data() + r.rec;
        for (int k = 0; k < r.nr; k++) {
            const int s1 = (int)(b[k] & 0xFFFFu), s2 = (int)(int16_t)(b[k] >> 16);
            // flux records read gradients (core and ring-1 cells); the others only states
            const int lim = k < r.ncc ? r.ncore : k < r.nrc ? ngrad : ncell;
            if (s1 >= lim || s2 >= lim || s2 < -4 || (k < r.ncc && s2 < 0)) return fail(t, "record slot");
            if (k < r.nrc && (k < r.nint) != (s2 >= 0)) return fail(t, "interior / boundary flux records");
            if (s2 < 0 && k >= r.ngeo) return fail(t, "boundary record without normal");
            if (s2 == -4) {
                const int q = T.qcell[r.rbase + k];
                if (q < 0 || q >= T.nc) return fail(t, "no-slip ghost cell");
            }
        }
        const uint16_t* off = T.csr.data() + r.csr;
        const uint16_t* ent = off + r.noff;   // entry e: ent[2e] (record << 1 | side), ent[2e + 1] other slot
        auto o = [&](int i) { return (int)(off[i] & 0x7FFF); };
        if (off[0] != 0 || 2 * o(ngrad) > r.ncsr - r.noff) return fail(t, "csr offsets");
        for (int g = 0; g < ngrad; g++) {
            if (o(g + 1) < o(g)) return fail(t, "csr offsets");
            const int c = g < r.ncore ? r.c0 + g : T.halo[r.halo + g - r.ncore];
            if (o(g + 1) - o(g) != L.inc_off[c + 1] - L.inc_off[c]) return fail(t, "csr row length");
            bool bcf = false;
            for (int e = o(g); e < o(g + 1); e++) bcf = bcf || (int16_t)ent[2 * e + 1] < 0;
            if (bcf != ((off[g + 1] & 0x8000) != 0)) return fail(t, "csr boundary flag");
            for (int e = o(g); e < o(g + 1); e++) {
                const int rr = ent[2 * e] >> 1, side = ent[2 * e] & 1, other = (int)(int16_t)ent[2 * e + 1];
                if (rr >= r.nr || (g < r.ncore && rr >= r.nrc)) return fail(t, "csr entry");
                const uint32_t sl = b[rr];
                const int s1 = (int)(sl & 0xFFFFu), s2 = (int)(int16_t)(sl >> 16);
                if ((side ? s2 : s1) != g || other != (side ? s1 : s2)) return fail(t, "csr entry slots");
            }
        }
    }
    if (cells != T.nc) { err = "tiles do not cover the cells"; return false; }
    return true;
}

bool build_tile_layout(const HostMesh& m, const DeviceLayout& L, TileLayout& T, std::string& err) {
    T = TileLayout();
    const int nc = L.nc, nf = L.nf;
    T.nc = nc;
    T.nc4 = round_up(nc, 4);
    Marks mk(nc, nf);
    int stamp = 0;
    Tile t;
    // tiles are the renumbering's 256-cell Hilbert blocks; a block that exceeds a capacity (cells
    // with very many faces) is split in halves until it fits
    std::vector<std::pair<int, int>> todo;
    for (int c0 = nc - (nc - 1) % kTileCore - 1; c0 >= 0; c0 -= kTileCore) todo.push_back({c0, std::min(kTileCore, nc - c0)});
    long long recs = 0, r1 = 0, r2 = 0;
    while (!todo.empty()) {
        const auto [c0, n] = todo.back();
        todo.pop_back();
        if (make_tile(L, c0, n, stamp++, mk, t)) {
            append_tile(m, L, t, mk, T);
            recs += (long long)t.faces.size() - (long long)(t.faces.size() - t.nrc);
            r1 += (long long)t.ring1.size();
            r2 += (long long)t.ring2.size();
            continue;
        }
        if (n == 1) {
            err = "cell " + std::to_string(m.cell_new2old[c0] + 1) + " and its neighbours exceed a tile's capacity";
            return false;
        }
        const int h = n / 2;
        todo.push_back({c0 + h, n - h});   // processed after the first half: tiles stay in cell order
        todo.push_back({c0, h});
    }
    if (!check_tile_layout(T, L, err)) return false;
    T.rec_per_face = nf ? (double)recs / nf : 0.0;
    T.ring1_per_cell = nc ? (double)r1 / nc : 0.0;
    T.ring2_per_cell = nc ? (double)r2 / nc : 0.0;
    T.vol.assign(T.nc4, 1.0f); T.rvol.assign(T.nc4, 1.0f);
    T.lsq.assign(T.nc4, std::array<float, 4>{0.f, 0.f, 0.f, 0.f});
    for (int c = 0; c < nc; c++) {
        T.vol[c] = (float)L.vol[c];
        T.rvol[c] = (float)(1.0 / L.vol[c]);
        T.lsq[c] = {(float)L.Ixx[c], (float)L.Iyy[c], (float)L.Ixy[c], 0.f};
    }
    return true;
}

}  // namespace fv2d
