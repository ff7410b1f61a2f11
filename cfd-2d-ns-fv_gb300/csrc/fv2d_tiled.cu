// FP32 engine: state, gradients and fluxes in FP32 (the LSQ moments stay FP64, the residual norms
// are accumulated in FP64), one fused kernel per SSP-RK3 stage over the tile layout
// (fv2d_tiles.h, fv2d_tiled.cuh).  A single solve (TiledSolver, the Solver interface) and a batch of
// independent solves (TiledBatch, the Batch interface) run on the same core and the same kernels,
// so a solve gives the same bits alone and in a batch; FMA contraction is therefore allowed here.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "fv2d_batch.h"
#include "fv2d_hostcopy.h"
#include "fv2d_range_alloc.h"
#include "fv2d_solver.h"
#include "fv2d_tiled.cuh"

namespace fv2d {

namespace {

#define FV2D_T(call)                                                                            \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            err = std::string(#call) + ": " + cudaGetErrorString(e_);                           \
            return e_ == cudaErrorMemoryAllocation ? FV2D_ERR_NOMEM : FV2D_ERR_CUDA;            \
        }                                                                                       \
    } while (0)

inline long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

// A mesh's tile layout in page-locked memory, built on its first admission and cached on the mesh.
struct TiledImage {
    std::vector<TileRec> tiles;
    std::vector<int> n2o;
    long long nc = 0, nc4 = 0, recw = 0, nrec = 0, ncsr = 0, nhalo = 0;
    double rec_per_face = 0, ring1 = 0, ring2 = 0;
    char* pin = nullptr;
    size_t o_rec = 0, o_qc = 0, o_csr = 0, o_halo = 0, o_vol = 0, o_rvol = 0, o_lsq = 0;
    ~TiledImage() { if (pin) cudaFreeHost(pin); }
};

int tiled_image(const HostMesh& hm, std::shared_ptr<TiledImage>& out, std::string& err) {
    auto& slot = hm.batch_image[1];
    if (slot) { out = std::static_pointer_cast<TiledImage>(slot); return FV2D_OK; }
    DeviceLayout D;
    build_layout(hm, D);
    TileLayout L;
    if (!build_tile_layout(hm, D, L, err)) return FV2D_ERR_MESH;
    auto im = std::make_shared<TiledImage>();
    im->nc = L.nc; im->nc4 = L.nc4; im->recw = (long long)L.rec.size(); im->nrec = (long long)L.qcell.size();
    im->ncsr = (long long)L.csr.size(); im->nhalo = (long long)L.halo.size();
    im->rec_per_face = L.rec_per_face; im->ring1 = L.ring1_per_cell; im->ring2 = L.ring2_per_cell;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
    im->o_rec = take(4 * L.rec.size()); im->o_qc = take(4 * L.qcell.size()); im->o_csr = take(2 * L.csr.size());
    im->o_halo = take(4 * L.halo.size()); im->o_vol = take(4 * (size_t)L.nc4); im->o_rvol = take(4 * (size_t)L.nc4);
    im->o_lsq = take(16 * (size_t)L.nc4);
    FV2D_T(cudaMallocHost(&im->pin, off));
    auto cp = [&](size_t o, const void* src, size_t bytes) { if (bytes) std::memcpy(im->pin + o, src, bytes); };
    cp(im->o_rec, L.rec.data(), 4 * L.rec.size()); cp(im->o_qc, L.qcell.data(), 4 * L.qcell.size());
    cp(im->o_csr, L.csr.data(), 2 * L.csr.size()); cp(im->o_halo, L.halo.data(), 4 * L.halo.size());
    cp(im->o_vol, L.vol.data(), 4 * (size_t)L.nc4); cp(im->o_rvol, L.rvol.data(), 4 * (size_t)L.nc4);
    cp(im->o_lsq, L.lsq.data(), 16 * (size_t)L.nc4);
    im->tiles = std::move(L.tiles);
    im->n2o = hm.cell_new2old;
    slot = im;
    out = im;
    return FV2D_OK;
}

}  // namespace

// Arena capacities of the core.
struct TiledCaps {
    long long cells = 0, recw = 0, recs = 0, csr = 0, halo = 0, tiles = 0;
    int solves = 0;
};

// Capacities for up to `cells` cells and `faces` faces in `solves` solves, with the per-face and
// per-cell allowances of the tile layout (Voronoi meshes use about 10.6 record words and 1.45
// records per face, 10 csr words and 0.8 halo ids per cell; the allowances leave room for smaller
// tiles and padding).
TiledCaps tiled_caps(long long cells, long long faces, int solves) {
    TiledCaps c;
    c.solves = solves;
    c.tiles = cells / 64 + 2LL * solves + 16;
    c.cells = round_up(cells + 4LL * solves, 4);
    c.recw = round_up(12 * faces + 32 * c.tiles, 4);
    c.recs = 2 * faces + 4 * c.tiles;
    // u16 words: offsets (~1.4 per cell) and two words per entry (~2.8 entries per face: both
    // incidences of a face, for core and ring-1 cells); measured 17.6 per cell on Voronoi meshes
    // (F = 3N), 11.4 on quads
    c.csr = round_up(6 * faces + 2 * cells + 16 * c.tiles, 8);
    c.halo = round_up(cells + cells / 2 + 4 * c.tiles, 4);
    return c;
}

// Device bytes of those capacities (per-cell state and geometry, tile blocks, descriptors).
long long tiled_bytes(const TiledCaps& c, bool keep_r) {
    const long long q4 = 16;
    long long b = c.cells * (3 * q4 + 6 * q4 + 2 * q4 + (keep_r ? q4 : 0) + 4 * 4 + 16);
    b += 4 * c.recw + 4 * c.recs + 2 * c.csr + 4 * c.halo;
    b += (long long)sizeof(TileDesc) * c.tiles + 40LL * c.tiles;    // descriptors, norm partials
    b += (long long)c.solves * ((long long)sizeof(TParams) + 4 + 4 + 32 + 8);
    return b + 64 * 1024;
}

class TiledCore {
public:
    struct Solve {
        bool active = false, need_init = false;
        long long c0 = 0, n = 0, n4 = 0, rw0 = 0, rw = 0, q0 = 0, nq = 0, cs0 = 0, ncs = 0, h0 = 0, nh = 0;
        int first_tile = 0, ntiles = 0, iterations = 0;
        int fpw = 32;   // flux records a warp takes per grab in this solve's tiles
        std::shared_ptr<TiledImage> image;
    };

    ~TiledCore() {
        if (stream_) cudaStreamSynchronize(stream_);
        drop_graphs();
        for (auto& p : pending_) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
        for (auto e : free_events_) cudaEventDestroy(e);
        if (arena_) cudaFree(arena_);
        if (desc_pin_) cudaFreeHost(desc_pin_);
        if (pin_params_) cudaFreeHost(pin_params_);
        if (stream_) cudaStreamDestroy(stream_);
    }

    int init(const TiledCaps& c, bool keep_r, bool norms) {
        caps_ = c;
        keep_r_ = keep_r;
        norms_ = norms;
        FV2D_T(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
        FV2D_T(cudaMallocHost(&pin_params_, sizeof(TParams) * (size_t)c.solves));
        // page-locked mirrors of the tile descriptors, the per-solve tile ranges and the tile count:
        // a solve's admission or removal copies only its own part
        FV2D_T(cudaMallocHost(&desc_pin_, sizeof(TileDesc) * (size_t)c.tiles + 8 * (size_t)c.solves + 64));
        sr_pin_ = (int*)((char*)desc_pin_ + sizeof(TileDesc) * (size_t)c.tiles);
        cnt_pin_ = sr_pin_ + 2 * (size_t)c.solves;
        std::memset(desc_pin_, 0, sizeof(TileDesc) * (size_t)c.tiles + 8 * (size_t)c.solves + 64);
        size_t off = 0;
        auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
        const size_t q4 = sizeof(Q4<float>), nc = (size_t)c.cells;
        size_t oq[3], og[3];
        for (int i = 0; i < 3; i++) oq[i] = take(q4 * nc);
        for (int i = 0; i < 3; i++) og[i] = take(2 * q4 * nc);
        const size_t oD = take(q4 * nc), olo = take(q4 * nc), oR = keep_r ? take(q4 * nc) : 0;
        const size_t odt = take(4 * nc), oS = take(4 * nc), ovol = take(4 * nc), orvol = take(4 * nc);
        const size_t olsq = take(16 * nc);
        const size_t orec = take(4 * (size_t)c.recw), oqc = take(4 * (size_t)c.recs), ocsr = take(2 * (size_t)c.csr);
        const size_t ohalo = take(4 * (size_t)c.halo);
        const size_t otiles = take(sizeof(TileDesc) * (size_t)c.tiles), otpart = take(32 * (size_t)c.tiles);
        const size_t oP = take(sizeof(TParams) * (size_t)c.solves), osmax = take(4 * (size_t)c.solves);
        const size_t oflag = take(4 * (size_t)c.solves), ores = take(32 * (size_t)c.solves);
        const size_t osr = take(8 * (size_t)c.solves), omisc = take(256);
        bytes_ = off;
        FV2D_T(cudaMalloc(&arena_, bytes_));
        char* a = (char*)arena_;
        for (int i = 0; i < 3; i++) { A_.Q[i] = (Q4<float>*)(a + oq[i]); A_.G[i] = (Q4<float>*)(a + og[i]); }
        A_.D = (Q4<float>*)(a + oD); A_.Qlo = (Q4<float>*)(a + olo); A_.R = keep_r ? (Q4<float>*)(a + oR) : nullptr;
        A_.dt = (float*)(a + odt); A_.S = (float*)(a + oS); A_.vol = (float*)(a + ovol); A_.rvol = (float*)(a + orvol);
        A_.lsq = (float4*)(a + olsq);
        A_.rec = (uint32_t*)(a + orec); A_.qcell = (int*)(a + oqc); A_.csr = (uint16_t*)(a + ocsr); A_.halo = (int*)(a + ohalo);
        A_.tiles = (TileDesc*)(a + otiles);
        A_.tpart = norms ? (double*)(a + otpart) : nullptr;
        A_.P = (TParams*)(a + oP); A_.smax = (float*)(a + osmax); A_.flags = (int*)(a + oflag);
        res2_ = (double*)(a + ores); srange_ = (int*)(a + osr);
        int* misc = (int*)(a + omisc);
        A_.ntiles = misc; A_.counter = misc + 4; A_.err = misc + 8;
        A_.store_r = 0;
        A_.nsmax = c.solves;
        FV2D_T(cudaMemsetAsync(arena_, 0, bytes_, stream_));
        FV2D_T(cudaStreamSynchronize(stream_));
        cells_.reset(c.cells); recw_.reset(c.recw); recs_.reset(c.recs); csr_.reset(c.csr); halo_.reset(c.halo);
        tiles_.reset(c.tiles);
        solves_.assign(c.solves, Solve());
        int dev = 0;
        FV2D_T(cudaGetDevice(&dev));
        FV2D_T(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev));
        FV2D_T(cudaFuncSetAttribute(k_tstage<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmTotal));
        FV2D_T(cudaFuncSetAttribute(k_tstage<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmTotal));
        FV2D_T(cudaFuncSetAttribute(k_tstage<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmTotal));
        int per = 0;
        FV2D_T(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_tstage<1>, kTileCore, kSmTotal));
        grid_ = std::max(1, per) * sms_;
        return FV2D_OK;
    }

    // Solve parameters (main.cpp:75-118, class_flow.hpp); fresh/init_prims as on creation.
    static TParams params(const fv2d_case& cs) {
        TParams p{};
        const double gm1 = cs.gamma - 1, Cp = cs.R * cs.gamma / (cs.gamma - 1), kc = (cs.mu * Cp) / cs.Pr;
        const double E = (cs.P / (cs.gamma - 1)) + 0.5 * cs.rho * (cs.u * cs.u + cs.v * cs.v);
        p.k.gamma = (float)cs.gamma; p.k.gm1 = (float)gm1; p.k.R = (float)cs.R; p.k.mu = (float)cs.mu; p.k.k = (float)kc;
        p.k.q_inf[0] = (float)cs.rho; p.k.q_inf[1] = (float)(cs.rho * cs.u); p.k.q_inf[2] = (float)(cs.rho * cs.v);
        p.k.q_inf[3] = (float)E;
        p.k.rho_inf = (float)cs.rho; p.k.u_inf = (float)cs.u; p.k.v_inf = (float)cs.v; p.k.P_inf = (float)cs.P;
        p.k.two_cfl = (float)(2 * cs.cfl);
        p.k.vn0 = (float)std::sqrt(cs.v * cs.v + cs.u * cs.u);
        p.k.c0 = (float)std::sqrt(cs.gamma * (cs.P / cs.rho));
        p.k.roe = cs.flux_solver == FV2D_ROE;
        p.order2 = cs.order == 2; p.ns = cs.eqn == FV2D_NS; p.squeeze = cs.limiter == FV2D_LIM_SQUEEZE;
        p.global_dt = cs.time_type == FV2D_DT_GLOBAL; p.fresh = 1; p.init_prims = 1;
        return p;
    }

    int add(const HostMesh& hm, const fv2d_case& cs, int* sid_out, int fpw = 32) {
        if (hm.bc1 != cs.bc1 || hm.bc2 != cs.bc2) { err = "mesh was built with other BC codes than this case"; return FV2D_ERR_ARG; }
        int sid = -1;
        for (int i = 0; i < caps_.solves; i++) if (!solves_[i].active) { sid = i; break; }
        if (sid < 0) { err = "batch is full (max solves)"; return FV2D_ERR_NOMEM; }
        std::shared_ptr<TiledImage> im;
        int rc = tiled_image(hm, im, err);
        if (rc) return rc;
        Solve s;
        s.n = im->nc; s.n4 = im->nc4; s.rw = im->recw; s.nq = im->nrec; s.ncs = im->ncsr; s.nh = im->nhalo;
        s.ntiles = (int)im->tiles.size();
        s.fpw = fpw;
        long long t0 = 0;
        if (!tiles_.alloc(s.ntiles, &t0)) { err = "batch tile capacity exhausted"; return FV2D_ERR_NOMEM; }
        s.first_tile = (int)t0;
        if (!cells_.alloc(s.n4, &s.c0)) { tiles_.release(t0, s.ntiles); err = "batch cell capacity exhausted"; return FV2D_ERR_NOMEM; }
        if (!recw_.alloc(s.rw, &s.rw0)) { release(s, 1); err = "batch record capacity exhausted"; return FV2D_ERR_NOMEM; }
        if (!recs_.alloc(s.nq, &s.q0)) { release(s, 2); err = "batch record capacity exhausted"; return FV2D_ERR_NOMEM; }
        if (!csr_.alloc(s.ncs, &s.cs0)) { release(s, 3); err = "batch csr capacity exhausted"; return FV2D_ERR_NOMEM; }
        if (!halo_.alloc(s.nh, &s.h0)) { release(s, 4); err = "batch halo capacity exhausted"; return FV2D_ERR_NOMEM; }
        // asynchronous copies from the page-locked image (kept alive by the solve record)
        const char* P = im->pin;
        auto up = [&](void* dst, size_t o, size_t bytes) {
            return bytes ? cudaMemcpyAsync(dst, P + o, bytes, cudaMemcpyHostToDevice, stream_) : cudaSuccess;
        };
        FV2D_T(up((void*)(A_.rec + s.rw0), im->o_rec, 4 * (size_t)s.rw));
        FV2D_T(up((void*)(A_.qcell + s.q0), im->o_qc, 4 * (size_t)s.nq));
        FV2D_T(up((void*)(A_.csr + s.cs0), im->o_csr, 2 * (size_t)s.ncs));
        FV2D_T(up((void*)(A_.halo + s.h0), im->o_halo, 4 * (size_t)s.nh));
        FV2D_T(up((float*)A_.vol + s.c0, im->o_vol, 4 * (size_t)s.n4));
        FV2D_T(up((float*)A_.rvol + s.c0, im->o_rvol, 4 * (size_t)s.n4));
        FV2D_T(up((void*)(A_.lsq + s.c0), im->o_lsq, 16 * (size_t)s.n4));
        pin_params_[sid] = params(cs);   // a slot is rewritten only after its solve was removed (synchronised)
        FV2D_T(cudaMemcpyAsync(A_.P + sid, pin_params_ + sid, sizeof(TParams), cudaMemcpyHostToDevice, stream_));
        // the uniform freestream state (main.cpp:75-118): hi = the state rounded to FP32, lo = the remainder
        const double E = (cs.P / (cs.gamma - 1)) + 0.5 * cs.rho * (cs.u * cs.u + cs.v * cs.v);
        const double qd[4] = {cs.rho, cs.rho * cs.u, cs.rho * cs.v, E};
        Q4<float> hi, lo;
        for (int j = 0; j < 4; j++) { hi.p[j] = (float)qd[j]; lo.p[j] = (float)(qd[j] - (double)hi.p[j]); }
        fill(s, hi, lo);
        FV2D_T(cudaGetLastError());
        FV2D_T(cudaMemsetAsync(A_.flags + sid, 0, 4, stream_));
        // the tile slots' norm partials (a previous occupant's): zero until this solve's first iteration
        if (A_.tpart && s.ntiles)
            FV2D_T(cudaMemsetAsync(A_.tpart + 4 * (size_t)s.first_tile, 0, 32 * (size_t)s.ntiles, stream_));
        s.need_init = true;          // spectral sums before the next step
        s.image = im;
        s.active = true;
        solves_[sid] = std::move(s);
        rc = put_tiles(sid, true);
        if (rc) return rc;
        *sid_out = sid;
        return FV2D_OK;
    }

    int remove(int sid) {
        if (sid < 0 || sid >= caps_.solves || !solves_[sid].active) { err = "no such solve"; return FV2D_ERR_ARG; }
        FV2D_T(cudaStreamSynchronize(stream_));
        Solve& s = solves_[sid];
        s.active = false;
        int rc = put_tiles(sid, false);   // empty descriptors: the kernels skip these tiles
        if (rc) return rc;
        release(s, 5);
        s = Solve();
        return FV2D_OK;
    }

    // The spectral sums of newly admitted solves (before the next step).
    int prepare() {
        for (int sid = 0; sid < caps_.solves; sid++) {
            Solve& s = solves_[sid];
            if (!s.active || !s.need_init) continue;
            int rc = spectral_init(sid);
            if (rc) return rc;
        }
        return FV2D_OK;
    }

    int spectral_init(int sid) {
        Solve& s = solves_[sid];
        FV2D_T(cudaMemsetAsync(A_.smax + sid, 0, 4, stream_));
        if (s.ntiles > 0) {
            const int gr = std::min(s.ntiles, 8 * sms_);
            k_tspec_init<<<gr, kTileCore, 0, stream_>>>(A_.tiles, s.first_tile, s.ntiles, A_.rec, A_.csr, A_.P, A_.S, A_.smax);
            FV2D_T(cudaGetLastError());
        }
        s.need_init = false;
        return FV2D_OK;
    }

    // One stage kernel over every tile.
    int launch_stage(int st) {
        // (the stage's tile counter was zeroed by the previous stage's kernel; the GLOBAL-dt maxima
        // by the second stage's)
        timed(st, [&] {
            // persistent grid (CTAs that take tiles until none is left) or one CTA per tile slot
            const int gr = full_grid_ ? (int)std::max<long long>(1, hi_tiles_) : grid_;
            if (st == 0) k_tstage<0><<<gr, kTileCore, kSmTotal, stream_>>>(A_);
            else if (st == 1) k_tstage<1><<<gr, kTileCore, kSmTotal, stream_>>>(A_);
            else k_tstage<2><<<gr, kTileCore, kSmTotal, stream_>>>(A_);
        });
        FV2D_T(cudaGetLastError());
        return FV2D_OK;
    }

    // Per-solve residual sums of squares from the last stage's per-tile partials (fixed order), on
    // demand: the partials of a tile slot hold its last iteration's values (zero until then).
    int reduce_norms() {
        if (!norms_) return FV2D_OK;
        k_tres_norm<<<caps_.solves, 256, 0, stream_>>>(srange_, A_.tpart, res2_);
        FV2D_T(cudaGetLastError());
        return FV2D_OK;
    }

    static constexpr int kGraphIters = 4;   // iterations per replay of the longer graph
    void drop_graphs() {
        for (auto& g : graph_) if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    }
    // Capture `iters` whole iterations as one graph.
    int capture(int iters, cudaGraphExec_t* out) {
        cudaGraph_t g;
        FV2D_T(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        int rc = FV2D_OK;
        for (int it = 0; it < iters && !rc; it++)
            for (int st = 0; st < 3 && !rc; st++) rc = launch_stage(st);
        cudaError_t e = cudaStreamEndCapture(stream_, &g);
        if (rc) return rc;
        if (e != cudaSuccess) { err = std::string("graph capture: ") + cudaGetErrorString(e); return FV2D_ERR_CUDA; }
        e = cudaGraphInstantiate(out, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { *out = nullptr; err = std::string("graph instantiate: ") + cudaGetErrorString(e); return FV2D_ERR_CUDA; }
        return FV2D_OK;
    }

    // Whole iterations as CUDA-graph replays (captured once; the graphs read the tile list from
    // device memory, so solves join and leave without re-capture): runs of kGraphIters iterations
    // as one replay (fewer gaps between replays), the rest one iteration per replay.
    int iterations(int n, bool graphs) {
        int it = 0;
        while (it < n) {
            int k = 1;
            if (!graphs || timing_) {
                for (int st = 0; st < 3; st++) { int rc = launch_stage(st); if (rc) return rc; }
            } else {
                const int w = n - it >= kGraphIters ? 1 : 0;
                k = w ? kGraphIters : 1;
                if (!graph_[w]) { int rc = capture(k, &graph_[w]); if (rc) return rc; }
                FV2D_T(cudaGraphLaunch(graph_[w], stream_));
            }
            for (auto& s : solves_) if (s.active) s.iterations += k;
            it += k;
        }
        return FV2D_OK;
    }

    // A solve's history flags rewritten (restart / load paths): the limiter's fresh face history and
    // the initial primitives; -1 keeps a flag as it is on the device (the kernel of an iteration's
    // second stage clears both).
    int set_history(int sid, int fresh, int init_prims) {
        FV2D_T(cudaStreamSynchronize(stream_));   // the pinned slot may still be read by an earlier copy
        if (fresh >= 0) {
            pin_params_[sid].fresh = fresh;
            FV2D_T(cudaMemcpyAsync(&A_.P[sid].fresh, &pin_params_[sid].fresh, 4, cudaMemcpyHostToDevice, stream_));
        }
        if (init_prims >= 0) {
            pin_params_[sid].init_prims = init_prims;
            FV2D_T(cudaMemcpyAsync(&A_.P[sid].init_prims, &pin_params_[sid].init_prims, 4, cudaMemcpyHostToDevice, stream_));
        }
        return FV2D_OK;
    }

    // Device status: CUDA errors, a kernel's timeout / descriptor error, non-physical states.
    int check(int* flags_out, int nflags) {
        FV2D_T(cudaStreamSynchronize(stream_));
        int e = 0;
        FV2D_T(cudaMemcpy(&e, A_.err, 4, cudaMemcpyDeviceToHost));
        if (e & 2) { err = "a stage kernel's wait for its tile copies timed out"; return FV2D_ERR_CUDA; }
        if (e & 4) { err = "a tile descriptor is out of range"; return FV2D_ERR_CUDA; }
        if (flags_out && nflags > 0) FV2D_T(cudaMemcpy(flags_out, A_.flags, 4 * (size_t)nflags, cudaMemcpyDeviceToHost));
        return FV2D_OK;
    }

    // The stage kernels' tile counters zeroed (the stage sequence restarts at stage 0).
    int reset_counters() {
        FV2D_T(cudaMemsetAsync(A_.counter, 0, 12, stream_));
        return FV2D_OK;
    }

    // Tuning (results do not depend on it): a solve's flux records per warp grab, the grid mode.
    int set_fpw(int sid, int fpw) {
        solves_[sid].fpw = fpw;
        return put_tiles(sid, true);
    }
    void set_full_grid(bool full) {
        if (full != full_grid_) drop_graphs();
        full_grid_ = full;
    }

    void set_timing(bool on) {
        timing_ = on;
        for (int i = 0; i < 3; i++) { ms_[i] = 0; launches_[i] = 0; }
    }
    int kernel_times(double* ms, int* launches) {
        FV2D_T(cudaStreamSynchronize(stream_));
        for (auto& p : pending_) {
            float t = 0;
            cudaEventElapsedTime(&t, p.a, p.b);
            ms_[p.kid] += t; launches_[p.kid] += 1;
            free_events_.push_back(p.a); free_events_.push_back(p.b);
        }
        pending_.clear();
        for (int i = 0; i < 3; i++) { ms[i] = ms_[i]; launches[i] = launches_[i]; }
        return FV2D_OK;
    }

    TArgs A_{};
    double* res2_ = nullptr;
    std::vector<Solve> solves_;
    TiledCaps caps_;
    cudaStream_t stream_ = nullptr;
    size_t bytes_ = 0;
    int sms_ = 1, grid_ = 1;
    bool full_grid_ = false;
    long long hi_tiles_ = 0;   // descriptor slots in use (up to the last active solve's)
    std::string err;
    RangeAlloc cells_, recw_, recs_, csr_, halo_, tiles_;

private:
    void release(Solve& s, int upto) {
        if (upto >= 1) { cells_.release(s.c0, s.n4); tiles_.release(s.first_tile, s.ntiles); }
        if (upto >= 2) recw_.release(s.rw0, s.rw);
        if (upto >= 3) recs_.release(s.q0, s.nq);
        if (upto >= 4) csr_.release(s.cs0, s.ncs);
        if (upto >= 5) halo_.release(s.h0, s.nh);
    }

    void fill(const Solve& s, Q4<float> hi, Q4<float> lo);

    // A solve's tile descriptors (arena offsets = its ranges' starts + the layout's solve-local
    // offsets) written into its slots of the descriptor array, or zeroed (an empty tile, which the
    // kernels skip) on removal; with its tile range (norms) and the descriptor count the kernels scan.
    int put_tiles(int sid, bool active) {
        const Solve& s = solves_[sid];
        TileDesc* d = desc_pin_ + s.first_tile;
        for (int i = 0; i < s.ntiles; i++) {
            TileDesc& x = d[i];
            x = TileDesc{};
            if (!active) continue;
            const TileRec& r = s.image->tiles[i];
            x.rec = s.rw0 + r.rec; x.rbase = s.q0 + r.rbase; x.csr = s.cs0 + r.csr; x.halo = s.h0 + r.halo;
            x.cbase = (int)s.c0; x.c0 = (int)(s.c0 + r.c0);
            x.ncore = r.ncore; x.n1 = r.n1; x.n2 = r.n2;
            x.nrc = r.nrc; x.ngeo = r.ngeo; x.nr = r.nr; x.nrp = r.nrp; x.ngp = r.ngp;
            x.noff = r.noff; x.ncsr = r.ncsr; x.nhalo = r.nhalo; x.sid = sid; x.ncc = r.ncc; x.fpw = s.fpw; x.nint = r.nint;
        }
        sr_pin_[2 * sid] = s.first_tile;
        sr_pin_[2 * sid + 1] = active ? s.ntiles : 0;
        long long hi = 0;
        for (int k = 0; k < caps_.solves; k++)
            if (solves_[k].active) hi = std::max<long long>(hi, (long long)solves_[k].first_tile + solves_[k].ntiles);
        *cnt_pin_ = (int)hi;
        if (full_grid_ && hi != hi_tiles_) drop_graphs();
        hi_tiles_ = hi;
        if (s.ntiles)
            FV2D_T(cudaMemcpyAsync((void*)(A_.tiles + s.first_tile), d, sizeof(TileDesc) * (size_t)s.ntiles,
                                   cudaMemcpyHostToDevice, stream_));
        FV2D_T(cudaMemcpyAsync(srange_ + 2 * sid, sr_pin_ + 2 * sid, 8, cudaMemcpyHostToDevice, stream_));
        FV2D_T(cudaMemcpyAsync((void*)A_.ntiles, cnt_pin_, 4, cudaMemcpyHostToDevice, stream_));
        // the count's mirror and this range are rewritten by later admissions or removals
        FV2D_T(cudaStreamSynchronize(stream_));
        return FV2D_OK;
    }

    template <class F>
    void timed(int kid, F&& fn) {
        if (!timing_) { fn(); return; }
        Pending p{kid, ev(), ev()};
        cudaEventRecord(p.a, stream_);
        fn();
        cudaEventRecord(p.b, stream_);
        pending_.push_back(p);
    }
    cudaEvent_t ev() {
        if (!free_events_.empty()) { cudaEvent_t e = free_events_.back(); free_events_.pop_back(); return e; }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
    struct Pending { int kid; cudaEvent_t a, b; };

    void* arena_ = nullptr;
    int* srange_ = nullptr;
    bool keep_r_ = false, norms_ = false, timing_ = false;
    cudaGraphExec_t graph_[2] = {nullptr, nullptr};   // one iteration, kGraphIters iterations
    TileDesc* desc_pin_ = nullptr;   // page-locked mirrors: descriptors, tile ranges, tile count
    int* sr_pin_ = nullptr;
    int* cnt_pin_ = nullptr;
    TParams* pin_params_ = nullptr;
    std::vector<Pending> pending_;
    std::vector<cudaEvent_t> free_events_;
    double ms_[3] = {0, 0, 0};
    int launches_[3] = {0, 0, 0};
};

namespace {
__global__ void k_tfill(Q4<float>* __restrict__ Q, Q4<float>* __restrict__ Qlo, int n, Q4<float> hi, Q4<float> lo) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        Q[i] = hi;
        Qlo[i] = lo;
    }
}
}  // namespace

void TiledCore::fill(const Solve& s, Q4<float> hi, Q4<float> lo) {
    const int gr = (int)std::min<long long>((s.n4 + 255) / 256, 4LL * sms_);
    k_tfill<<<std::max(gr, 1), 256, 0, stream_>>>(A_.Q[0] + s.c0, A_.Qlo + s.c0, (int)s.n4, hi, lo);
}

#undef FV2D_T
#define FV2D_T(call)                                                                            \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            err_ = std::string(#call) + ": " + cudaGetErrorString(e_);                          \
            return e_ == cudaErrorMemoryAllocation ? FV2D_ERR_NOMEM : FV2D_ERR_CUDA;            \
        }                                                                                       \
    } while (0)

// ------------------------------------------------------------------------------------------
// One solve (the Solver interface): stage-by-stage or graph-replayed iterations, state and field
// transfers in the reference's numbering, the residual kept for norms and output.
class TiledSolver : public Solver {
public:
    ~TiledSolver() override {
        if (host_stage_) cudaFreeHost(host_stage_);
        for (cudaEvent_t e : copy_events_) cudaEventDestroy(e);
        if (stage_free_) cudaEventDestroy(stage_free_);
        if (dstage_) cudaFree(dstage_);
    }

    int init(const fv2d_case& cs) override {
        cs_ = cs;
        nc_ = mesh_.nc;
        order2_ = cs.order == 2;
        std::shared_ptr<TiledImage> im;
        int rc = tiled_image(mesh_, im, err_);
        if (rc) return rc;
        TiledCaps c;
        c.cells = im->nc4; c.recw = im->recw; c.recs = im->nrec; c.csr = im->ncsr; c.halo = std::max<long long>(4, im->nhalo);
        c.tiles = (long long)im->tiles.size(); c.solves = 1;
        rc = core_.init(c, true, false);
        if (rc) { err_ = core_.err; return rc; }
        rc = core_.add(mesh_, cs, &sid_);
        if (rc) { err_ = core_.err; return rc; }
        rc = core_.prepare();
        if (rc) { err_ = core_.err; return rc; }
        n2o_ = im->n2o;
        // one allocation: field staging (8 doubles per cell), the cell permutation and the norm
        // partials, each region starting on a 256-byte boundary
        size_t off = 0;
        auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
        take(8 * 8 * (size_t)nc_);
        const size_t o_n2o = take(4 * (size_t)nc_), o_part = take(32 * 304);
        FV2D_T(cudaMalloc(&dstage_, off));
        dn2o_ = (int*)((char*)dstage_ + o_n2o);
        part_ = (double*)((char*)dstage_ + o_part);
        staging_bytes_ = std::max<size_t>(8 * 8 * (size_t)nc_, 32 * 304);
        FV2D_T(cudaMallocHost(&host_stage_, staging_bytes_));
        FV2D_T(cudaEventCreateWithFlags(&stage_free_, cudaEventDisableTiming));
        std::memcpy(host_stage_, n2o_.data(), 4 * (size_t)nc_);
        FV2D_T(cudaMemcpyAsync(dn2o_, host_stage_, 4 * (size_t)nc_, cudaMemcpyHostToDevice, core_.stream_));
        FV2D_T(cudaStreamSynchronize(core_.stream_));
        stage_ = 0;
        last_stage_ = -1;
        return FV2D_OK;
    }

    int stage() override {
        const int s = stage_;
        int rc = core_.launch_stage(s);
        if (rc) { err_ = core_.err; return rc; }
        last_stage_ = s;
        stage_ = (s + 1) % 3;
        return FV2D_OK;
    }

    int step(int iterations) override {
        if (iterations < 0) { err_ = "negative iteration count"; return FV2D_ERR_ARG; }
        int rc, done = 0;
        if (stage_ != 0) {
            while (stage_ != 0) if ((rc = stage())) return rc;
            done = 1;
        }
        if (iterations > done) {
            rc = core_.iterations(iterations - done, graphs_ && !store_every_);
            if (rc) { err_ = core_.err; return rc; }
            last_stage_ = 2;
        }
        return FV2D_OK;
    }

    int set_state(const double* q) override {
        int rc = upload(q);
        if (rc) return rc;
        rc = core_.set_history(sid_, 1, 0);   // restart: fresh face histories, primitives from the state
        if (!rc) rc = core_.spectral_init(sid_);
        if (!rc && stage_ != 0) rc = core_.reset_counters();   // the stage sequence restarts
        if (rc) { err_ = core_.err; return rc; }
        stage_ = 0;
        return FV2D_OK;
    }

    int load_state(const double* q) override {
        if (stage_ != 0) { err_ = "load_state between iterations only (stage counter is not 0)"; return FV2D_ERR_ARG; }
        int rc = upload(q);
        if (rc) return rc;
        rc = core_.set_history(sid_, -1, 0);
        if (rc) { err_ = core_.err; return rc; }
        return FV2D_OK;
    }

    int get_field(int field, double* out) override {
        int rc = synchronize();
        if (rc && rc != FV2D_ERR_STATE) return rc;
        const TArgs& A = core_.A_;
        const long long c0 = core_.solves_[sid_].c0;
        const void* src = nullptr;
        int ncomp = 4;
        switch (field) {
            case FV2D_F_QBAR: src = A.Q[0] + c0; break;
            case FV2D_F_QSTAR: src = (last_stage_ == 0 ? A.Q[1] : A.Q[2]) + c0; break;
            case FV2D_F_RES: src = A.R + c0; break;
            case FV2D_F_DT: src = A.dt + c0; ncomp = 1; break;
            case FV2D_F_QBAR_GRAD: src = A.G[0] + 2 * c0; ncomp = 8; break;
            case FV2D_F_QSTAR_GRAD:
                ncomp = 8;
                if (last_stage_ <= 0 || !order2_) { std::fill(out, out + 8 * (size_t)nc_, 0.0); return FV2D_OK; }
                src = A.G[last_stage_] + 2 * c0;
                break;
            default: {
                const int n = mesh_field(mesh_, field, out);
                if (n < 0) { err_ = "unknown field id"; return FV2D_ERR_ARG; }
                return FV2D_OK;
            }
        }
        if (field == FV2D_F_QBAR_GRAD && !order2_) { std::fill(out, out + 8 * (size_t)nc_, 0.0); return FV2D_OK; }
        cudaStream_t st = core_.stream_;
        if (ncomp == 1)
            k_scalar_out<float><<<(nc_ + 255) / 256, 256, 0, st>>>(nc_, dn2o_, (const float*)src, dstage_);
        else
            k_state_out<float><<<(nc_ + 255) / 256, 256, 0, st>>>(nc_, ncomp, dn2o_, (const Q4<float>*)src, dstage_,
                                                                   field == FV2D_F_QBAR ? A.Qlo + c0 : nullptr);
        FV2D_T(cudaGetLastError());
        FV2D_T(staged_d2h(out, dstage_, 8 * (size_t)ncomp * nc_, host_stage_, st, copy_events_));
        return rc;
    }

    int residual_norm(double out[4]) override {
        cudaStream_t st = core_.stream_;
        k_res_norm_partial<float><<<304, 256, 0, st>>>(nc_, core_.A_.R + core_.solves_[sid_].c0, part_);
        FV2D_T(cudaGetLastError());
        FV2D_T(cudaMemcpyAsync(host_stage_, part_, 32 * 304, cudaMemcpyDeviceToHost, st));
        int rc = synchronize();
        const double* p = (const double*)host_stage_;
        double acc[4] = {0, 0, 0, 0};
        for (int b = 0; b < 304; b++) for (int j = 0; j < 4; j++) acc[j] += p[4 * b + j];
        for (int j = 0; j < 4; j++) out[j] = std::sqrt(acc[j]);
        return rc;
    }

    int synchronize() override {
        int flag = 0;
        int rc = core_.check(&flag, 1);
        if (rc) { err_ = core_.err; return rc; }
        if (flag) { err_ = "non-physical state (rho <= 0, E <= 0 or NaN) produced by an update"; return FV2D_ERR_STATE; }
        return FV2D_OK;
    }

    int set_store_residual(int every) override {
        store_every_ = every != 0;
        core_.A_.store_r = store_every_ ? 1 : 0;
        return FV2D_OK;
    }
    int set_graphs(int enable) override { graphs_ = enable != 0; return FV2D_OK; }
    int set_timing(int enable) override { core_.set_timing(enable != 0); return FV2D_OK; }
    int kernel_times(double* ms, int* launches) override {
        for (int i = 0; i < K_COUNT; i++) { ms[i] = 0; launches[i] = 0; }
        double t[3];
        int l[3];
        int rc = core_.kernel_times(t, l);
        if (rc) { err_ = core_.err; return rc; }
        for (int i = 0; i < 3; i++) { ms[K_TSTAGE] += t[i]; launches[K_TSTAGE] += l[i]; }
        return FV2D_OK;
    }
    void* stream() override { return (void*)core_.stream_; }
    long long device_bytes() const override { return (long long)core_.bytes_; }

private:
    int upload(const double* q) {
        cudaStream_t st = core_.stream_;
        FV2D_T(staged_h2d(dstage_, q, 8 * 4 * (size_t)nc_, host_stage_, st, stage_free_));
        const long long c0 = core_.solves_[sid_].c0;
        k_state_in<float><<<(nc_ + 255) / 256, 256, 0, st>>>(nc_, dn2o_, dstage_, core_.A_.Q[0] + c0, core_.A_.Qlo + c0);
        FV2D_T(cudaGetLastError());
        return FV2D_OK;
    }

    TiledCore core_;
    fv2d_case cs_{};
    int sid_ = 0, nc_ = 0, last_stage_ = -1;
    bool order2_ = false, store_every_ = false, graphs_ = true;
    std::vector<int> n2o_;
    double* dstage_ = nullptr;
    int* dn2o_ = nullptr;
    double* part_ = nullptr;
    void* host_stage_ = nullptr;
    size_t staging_bytes_ = 0;
    std::vector<cudaEvent_t> copy_events_;
    cudaEvent_t stage_free_ = nullptr;
};

// ------------------------------------------------------------------------------------------
// Many solves (the Batch interface).
class TiledBatch : public Batch {
public:
    int init(long long max_cells, long long max_faces, int max_solves) override {
        if (max_cells <= 0 || max_faces <= 0 || max_solves <= 0 || max_cells > (1LL << 30) || max_faces > (1LL << 31)) {
            err_ = "batch capacity out of range (cells <= 2^30, faces <= 2^31)";
            return FV2D_ERR_ARG;
        }
        int rc = core_.init(tiled_caps(max_cells, max_faces, max_solves), false, true);
        if (rc) err_ = core_.err;
        return rc;
    }

    int add(const fv2d_mesh_desc* d, const fv2d_case* cs, int* sid) override {
        HostMesh hm;
        int rc = build_mesh(d, cs, hm, err_);
        if (rc) return rc;
        return add_mesh(hm, cs, sid);   // the solve keeps the mesh's page-locked image alive
    }

    int add_mesh(const HostMesh& hm, const fv2d_case* cs, int* sid) override {
        int rc = core_.add(hm, *cs, sid, fpw_for(hm.nc));
        if (rc) err_ = core_.err;
        return rc;
    }

    int remove(int sid) override {
        int rc = core_.remove(sid);
        if (rc) err_ = core_.err;
        return rc;
    }

    int step(int iterations) override {
        if (iterations < 0) { err_ = "negative iteration count"; return FV2D_ERR_ARG; }
        int rc = core_.prepare();
        if (!rc) rc = core_.iterations(iterations, true);
        if (rc) err_ = core_.err;
        return rc;
    }

    int norms(int* sids, double* out, int* iters, int max, int* n) override {
        int rc = core_.reduce_norms();
        if (rc) { err_ = core_.err; return rc; }
        rc = synchronize();
        std::vector<double> h(4 * (size_t)core_.caps_.solves);
        FV2D_T(cudaMemcpy(h.data(), core_.res2_, 32 * (size_t)core_.caps_.solves, cudaMemcpyDeviceToHost));
        int k = 0;
        for (int s = 0; s < core_.caps_.solves && k < max; s++) {
            if (!core_.solves_[s].active) continue;
            sids[k] = s;
            if (iters) iters[k] = core_.solves_[s].iterations;
            for (int j = 0; j < 4; j++) out[4 * k + j] = std::sqrt(h[4 * s + j]);
            k++;
        }
        *n = k;
        return rc;
    }

    int get_state(int sid, double* q) override {
        if (sid < 0 || sid >= core_.caps_.solves || !core_.solves_[sid].active) { err_ = "no such solve"; return FV2D_ERR_ARG; }
        const TiledCore::Solve& s = core_.solves_[sid];
        std::vector<Q4<float>> h(s.n), lo(s.n);
        FV2D_T(cudaStreamSynchronize(core_.stream_));
        FV2D_T(cudaMemcpy(h.data(), core_.A_.Q[0] + s.c0, sizeof(Q4<float>) * s.n, cudaMemcpyDeviceToHost));
        FV2D_T(cudaMemcpy(lo.data(), core_.A_.Qlo + s.c0, sizeof(Q4<float>) * s.n, cudaMemcpyDeviceToHost));
        const std::vector<int>& n2o = s.image->n2o;
        for (long long c = 0; c < s.n; c++)
            for (int j = 0; j < 4; j++) q[(size_t)j * s.n + n2o[c]] = (double)h[c].p[j] + (double)lo[c].p[j];
        int f = 0;
        FV2D_T(cudaMemcpy(&f, core_.A_.flags + sid, 4, cudaMemcpyDeviceToHost));
        if (f) { err_ = "non-physical state (rho <= 0, E <= 0 or NaN) in this solve"; return FV2D_ERR_STATE; }
        return FV2D_OK;
    }

    int synchronize() override {
        int rc = core_.check(nullptr, 0);
        if (rc) err_ = core_.err;
        return rc;
    }

    // The FP32 engine's tiles are fixed by its layout (up to 256 cells, one CTA of 256 threads per
    // tile); its tuning is, per solve-size bucket, the faces per warp of the flux pass (flux records a
    // warp takes per grab: 32 x tile_mult) and the grid mode (persistent CTAs, or one CTA per tile).
    // `block` is validated and kept but does not change the launch.
    int set_tuning(const BatchTuning& t) override {
        if (t.block < 64 || t.block > 256 || (t.block & 31)) { err_ = "block must be a multiple of 32 in [64, 256]"; return FV2D_ERR_ARG; }
        for (int b = 0; b < 3; b++) if (t.tile_mult[b] < 1 || t.tile_mult[b] > 32) { err_ = "tile multiple out of range [1, 32]"; return FV2D_ERR_ARG; }
        tune_ = t;
        core_.set_full_grid(t.full_grid != 0);
        for (int sid = 0; sid < core_.caps_.solves; sid++) {
            if (!core_.solves_[sid].active) continue;
            const int rc = core_.set_fpw(sid, fpw_for(core_.solves_[sid].n));
            if (rc) { err_ = core_.err; return rc; }
        }
        return FV2D_OK;
    }
    int fpw_for(long long cells) const {
        const int b = cells < tune_.bucket_edges[0] ? 0 : cells < tune_.bucket_edges[1] ? 1 : 2;
        return 32 * tune_.tile_mult[b];
    }
    BatchTuning tuning() const override { return tune_; }

    int usage(long long* o) override {
        long long act = 0;
        for (auto& s : core_.solves_) act += s.active;
        o[0] = core_.cells_.used(); o[1] = core_.cells_.cap(); o[2] = core_.recs_.used(); o[3] = core_.recs_.cap();
        o[4] = core_.csr_.used(); o[5] = core_.csr_.cap(); o[6] = act; o[7] = (long long)core_.bytes_;
        return FV2D_OK;
    }
    int set_timing(int enable) override { core_.set_timing(enable != 0); return FV2D_OK; }
    int kernel_times(double* ms, int* launches) override {
        int rc = core_.kernel_times(ms, launches);
        if (rc) err_ = core_.err;
        return rc;
    }
    void* stream() override { return (void*)core_.stream_; }

private:
    TiledCore core_;
    BatchTuning tune_;
};

#undef FV2D_T

Solver* make_solver_fp32() { return new TiledSolver(); }
Batch* make_batch_fp32() { return new TiledBatch(); }

void tiled_footprint(long long cells, long long faces, long long* bytes) {
    *bytes = tiled_bytes(tiled_caps(cells, faces, 1), false);
}

}  // namespace fv2d
