// Batched engine: many independent solves in one device arena.
//
// Every solve owns a contiguous cell range, face range and incidence range of the arena's
// capacity-sized arrays; its arrays hold ARENA ids (cell, face and incidence ids shifted by the
// range starts), so the per-element device functions of the single-solve kernels run unchanged.
// Work is described by tile lists in device memory (tile = up to `block * mult` cells or faces of
// one solve); each stage kernel is a persistent grid looping over its tiles, loads the solve's
// parameters into shared memory once per tile and applies the same per-element code.  One
// iteration (3 stages x 3 kernels + 2 memsets) is captured in a CUDA graph; since the graph reads
// the tile lists and parameter table from device memory, solves can join and leave between
// iterations without re-capturing.  Per-solve reductions: the GLOBAL dt maximum uses one atomic
// max per tile (a maximum does not depend on the order); the residual L2 sums are written per tile
// and summed per solve over its tiles in a fixed order (kb_res_norm), so they are reproducible bit
// for bit from run to run.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <vector>

#include "fv2d_batch.h"
#include "fv2d_kernels.cuh"
#include "fv2d_range_alloc.h"

namespace fv2d {

template <class T>
struct SolveParams {
    Consts<T> k;
    int order2, ns, squeeze, global_dt;
    int fresh, init_prims, pad0, pad1;
};

struct Tile {
    int sid, start, count, pad;
};

template <class T>
__device__ __forceinline__ T block_sum(T v, T* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    T s = T(0);
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += red[i];
    return s;   // valid in thread 0
}

template <class T>
__device__ __forceinline__ T block_max_t(T v, T* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max2(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    T s = T(0);
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) s = max2(s, red[i]);
    return s;   // valid in thread 0
}

#ifndef FV2D_BATCH_FVAL
#define FV2D_BATCH_FVAL 1   // FP64 batches store the face states for the limiter (0: recompute them)
#endif

// Largest block the batch kernels accept (the autotuner's largest) and the FP32 kernels' minimum
// resident blocks at that size (their register caps: gradient 64, face 48 - measured fastest);
// FP64 keeps a 128-register cap.
#ifndef FV2D_KB_MAXT
#define FV2D_KB_MAXT 256
#endif
#ifndef FV2D_KBG_MINB32
#define FV2D_KBG_MINB32 4
#endif
constexpr int kBatchMaxBlock = FV2D_KB_MAXT;
constexpr int kBatchMinB64 = 512 / FV2D_KB_MAXT;
#ifndef FV2D_KBG_MINB64
#define FV2D_KBG_MINB64 kBatchMinB64
#endif
template <class T>
__global__ void __launch_bounds__(FV2D_KB_MAXT, sizeof(T) == 4 ? FV2D_KBG_MINB32 : FV2D_KBG_MINB64)
kb_gradient(const Tile* __restrict__ tiles, const int* __restrict__ ntiles, DevMesh<T> m,
            const SolveParams<T>* __restrict__ P, const Q4<T>* __restrict__ Qin, const Q4<T>* __restrict__ Qprev,
            const Q4<T>* __restrict__ Gprev, Q4<T>* __restrict__ Gout) {
    __shared__ SolveParams<T> sp;
    __shared__ Tile st;
    const int nt = *ntiles;
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
        if (threadIdx.x == 0) { st = tiles[t]; sp = P[st.sid]; }
        __syncthreads();
        if (sp.order2) {
            if (sp.squeeze) {
                for (int e = threadIdx.x; e < st.count; e += blockDim.x)
                    gradient_cell<T, true, sizeof(T) == 8, FV2D_KB_MAXT / 32>(st.start + e, m, Qin, Qprev, Gprev, Gout, sp.k,
                                                                             sp.fresh, sp.init_prims);
            } else {
                for (int e = threadIdx.x; e < st.count; e += blockDim.x)
                    gradient_cell<T, false>(st.start + e, m, Qin, Qprev, Gprev, Gout, sp.k, sp.fresh, sp.init_prims);
            }
        }
        __syncthreads();
    }
}

#ifndef FV2D_KBF_MINB32
#define FV2D_KBF_MINB32 5
#endif
template <class T, bool LAST>
__global__ void __launch_bounds__(FV2D_KB_MAXT, sizeof(T) == 4 ? FV2D_KBF_MINB32 : kBatchMinB64)
kb_face(const Tile* __restrict__ tiles, const int* __restrict__ ntiles, DevMesh<T> m,
        const SolveParams<T>* __restrict__ P, const Q4<T>* __restrict__ Qin, const Q4<T>* __restrict__ G,
        Q4<T>* __restrict__ tout, T* __restrict__ sout) {
    __shared__ SolveParams<T> sp;
    __shared__ Tile st;
    const int nt = *ntiles;
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
        if (threadIdx.x == 0) { st = tiles[t]; sp = P[st.sid]; }
        __syncthreads();
        if (!sp.order2) {
            for (int e = threadIdx.x; e < st.count; e += blockDim.x)
                face_flux<T, false, false, LAST>(st.start + e, m, Qin, G, tout, sout, sp.k, sp.init_prims);
        } else if (sp.ns) {
            for (int e = threadIdx.x; e < st.count; e += blockDim.x)
                face_flux<T, true, true, LAST>(st.start + e, m, Qin, G, tout, sout, sp.k, sp.init_prims);
        } else {
            for (int e = threadIdx.x; e < st.count; e += blockDim.x)
                face_flux<T, true, false, LAST>(st.start + e, m, Qin, G, tout, sout, sp.k, sp.init_prims);
        }
        __syncthreads();
    }
}

template <class T, int STAGE>
__global__ void __launch_bounds__(FV2D_KB_MAXT)
kb_update(const Tile* __restrict__ tiles, const int* __restrict__ ntiles, DevMesh<T> m, SolveParams<T>* P,
          const Q4<T>* __restrict__ tface, const T* __restrict__ sface, Q4<T>* __restrict__ Qn, Q4<T>* __restrict__ Q1,
          Q4<T>* __restrict__ Q2, T* __restrict__ dt, T* __restrict__ S, T* __restrict__ smax, double* __restrict__ tpart,
          int* __restrict__ flags, Q4<T>* __restrict__ D, Q4<T>* __restrict__ Qlo) {
    __shared__ SolveParams<T> sp;
    __shared__ Tile st;
    __shared__ double redd[32];
    __shared__ T redt[32];
    const int nt = *ntiles;
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
        if (threadIdx.x == 0) { st = tiles[t]; sp = P[st.sid]; }
        __syncthreads();
        const T sm = (STAGE == 0 && sp.global_dt) ? smax[st.sid] : T(0);
        T mx = T(0);
        double acc[4] = {0, 0, 0, 0};
        for (int e = threadIdx.x; e < st.count; e += blockDim.x) {
            T r[4];
            const T sn = update_cell<T, STAGE>(st.start + e, m, tface, sface, Qn, Q1, Q2, dt, S, sm, nullptr,
                                               flags + st.sid, sp.k, sp.global_dt, r, D, Qlo);
            if (STAGE == 2) {
                mx = max2(mx, sn);
#pragma unroll
                for (int j = 0; j < 4; j++) acc[j] += (double)r[j] * (double)r[j];
            }
        }
        if (STAGE == 2) {
            const T bm = block_max_t(mx, redt);
            if (threadIdx.x == 0) atomic_max_pos(smax + st.sid, bm);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const double bs = block_sum(acc[j], redd);
                if (threadIdx.x == 0) tpart[4 * (size_t)t + j] = bs;   // this tile's sum of squares
            }
        }
        if (STAGE == 0 && threadIdx.x == 0) { P[st.sid].fresh = 0; P[st.sid].init_prims = 0; }
        __syncthreads();
    }
}

// Per-solve residual sums of squares: solve s owns the cell tiles [srange[2s], srange[2s] +
// srange[2s+1]) of the tile list; one block per solve slot adds their per-tile sums (kb_update,
// last stage) in a fixed order - a strided pass per thread, then the block's fixed-shape tree - so
// the result is the same bits on every run.  A slot without tiles gets zeros.  (A template only so
// that each precision's translation unit may include it.)
template <class T>
__global__ void __launch_bounds__(256)
kb_res_norm(const int* __restrict__ srange, const double* __restrict__ tpart, double* __restrict__ res2) {
    __shared__ double sh[4][256];
    const int s = blockIdx.x, first = srange[2 * s], n = srange[2 * s + 1];
    double acc[4] = {0, 0, 0, 0};
    for (int i = threadIdx.x; i < n; i += blockDim.x)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[j] += tpart[4 * (size_t)(first + i) + j];
#pragma unroll
    for (int j = 0; j < 4; j++) sh[j][threadIdx.x] = acc[j];
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
#pragma unroll
            for (int j = 0; j < 4; j++) sh[j][threadIdx.x] += sh[j][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0)
#pragma unroll
        for (int j = 0; j < 4; j++) res2[4 * s + j] = sh[j][0];
}

// A newly admitted solve's ids: solve-local -> arena (CSR offsets + i0, face ids + f0, cell ids + c0;
// negative BC codes and "no ghost cell" (-1) entries unchanged).
template <class I>   // I = int (a template so each precision's unit may include it)
__global__ void k_shift_ids(I* __restrict__ inc_off, int n1, I i0, I* __restrict__ inc, I* __restrict__ nbr, int k,
                            I* __restrict__ fc1, I* __restrict__ fc2, I* __restrict__ qcell, int m, I f0, I c0) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < max(n1, max(k, m)); i += gridDim.x * blockDim.x) {
        if (i < n1) inc_off[i] += i0;
        if (i < k) {
            const int v = inc[i];
            inc[i] = (((v >> 1) + f0) << 1) | (v & 1);
            if (nbr[i] >= 0) nbr[i] += c0;
        }
        if (i < m) {
            fc1[i] += c0;
            if (fc2[i] >= 0) fc2[i] += c0;
            if (qcell[i] >= 0) qcell[i] += c0;
        }
    }
}

// A newly admitted solve's uniform initial state (and its FP32 compensation term).
template <class T>
__global__ void k_fill_q(Q4<T>* __restrict__ Q, Q4<T>* __restrict__ Qlo, int n, Q4<T> hi, Q4<T> lo) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        Q[i] = hi;
        if (Qlo) Qlo[i] = lo;
    }
}

#define FV2D_B(call)                                                                              \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            err_ = std::string(#call) + ": " + cudaGetErrorString(e_);                            \
            return e_ == cudaErrorMemoryAllocation ? FV2D_ERR_NOMEM : FV2D_ERR_CUDA;              \
        }                                                                                         \
    } while (0)

template <class T>
class BatchImpl : public Batch {
    struct Rec {
        bool active = false;
        long long c0 = 0, n = 0, f0 = 0, m = 0, i0 = 0, k = 0;
        std::vector<int> n2o;
        int iterations = 0;
        std::shared_ptr<void> image;   // the mesh's upload image (source of in-flight copies)
    };

public:
    ~BatchImpl() override {
        if (stream_) cudaStreamSynchronize(stream_);   // copies from the solves' images may be in flight
        if (graph_) cudaGraphExecDestroy(graph_);
        for (auto& p : pending_) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
        for (auto e : free_events_) cudaEventDestroy(e);
        if (arena_) cudaFree(arena_);
        if (tile_pin_) cudaFreeHost(tile_pin_);
        if (pin_params_) cudaFreeHost(pin_params_);
        if (tiles_free_) cudaEventDestroy(tiles_free_);
        if (stream_) cudaStreamDestroy(stream_);
    }

    int init(long long max_cells, long long max_faces, int max_solves) override {
        if (max_cells <= 0 || max_faces <= 0 || max_solves <= 0 || max_cells > (1LL << 30) || max_faces > (1LL << 29)) {
            err_ = "batch capacity out of range (cells <= 2^30, faces <= 2^29)";
            return FV2D_ERR_ARG;
        }
        Nc_ = max_cells + max_solves;   // one sentinel offset slot per solve
        Fc_ = max_faces;
        Ic_ = 2 * max_faces;
        S_ = max_solves;
        FV2D_B(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
        FV2D_B(cudaEventCreateWithFlags(&tiles_free_, cudaEventDisableTiming));
        FV2D_B(cudaMallocHost(&pin_params_, sizeof(SolveParams<T>) * (size_t)max_solves));
        size_t off = 0;
        auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
        const size_t q4 = sizeof(Q4<T>);
        size_t oq[3], og[3];
        for (int i = 0; i < 3; i++) oq[i] = take(q4 * Nc_);
        for (int i = 0; i < 3; i++) og[i] = take(2 * q4 * Nc_);
        size_t odt = take(sizeof(T) * Nc_), oS = take(sizeof(T) * Nc_), ovol = take(sizeof(T) * Nc_);
        size_t orvol = take(sizeof(T) * Nc_), ordist = take(sizeof(T) * Fc_);
        size_t oixx = take(8 * Nc_), oiyy = take(8 * Nc_), oixy = take(8 * Nc_), ooff = take(4 * Nc_);
        size_t oinc = take(4 * Ic_), onbr = take(4 * Ic_), oigeo = take(q4 * Ic_);
        size_t ofc1 = take(4 * Fc_), ofc2 = take(4 * Fc_), oqc = take(4 * Fc_);
        size_t ogeo[14];
        for (int gI = 0; gI < 14; gI++) ogeo[gI] = take(sizeof(T) * Fc_);
        size_t ot = take(q4 * Fc_), os = take(sizeof(T) * Fc_);
        size_t oP = take(sizeof(SolveParams<T>) * S_), osmax = take(sizeof(T) * S_), ores = take(32 * (size_t)S_);
        size_t oflag = take(4 * (size_t)S_);
        const bool comp = sizeof(T) == 4;   // FP32: delta-form increments + compensated base state
        size_t oD = comp ? take(q4 * Nc_) : 0, olo = comp ? take(q4 * Nc_) : 0;
        // FP64: the face pass stores its reconstructed face states for the next squeeze (as the
        // single-solve FP64 engine does); a solve's first stage after admission uses the sentinel
        const bool fv = !comp && FV2D_BATCH_FVAL;
        size_t ofval = fv ? take(2 * q4 * Fc_) : 0;
        tile_cap_ = (int)std::min<long long>((Nc_ + Fc_) / 64 + 4 * (long long)S_ + 16, 1LL << 28);
        size_t otc = take(sizeof(Tile) * tile_cap_), otf = take(sizeof(Tile) * tile_cap_), ocnt = take(64);
        size_t otp = take(32 * (size_t)tile_cap_), osr = take(8 * (size_t)S_);
        bytes_ = off;
        FV2D_B(cudaMalloc(&arena_, bytes_));
        char* a = (char*)arena_;
        for (int i = 0; i < 3; i++) { Q_[i] = (Q4<T>*)(a + oq[i]); G_[i] = (Q4<T>*)(a + og[i]); }
        dt_ = (T*)(a + odt); S_arr_ = (T*)(a + oS);
        T* vol = (T*)(a + ovol);
        double *ixx = (double*)(a + oixx), *iyy = (double*)(a + oiyy), *ixy = (double*)(a + oixy);
        int *incoff = (int*)(a + ooff), *inc = (int*)(a + oinc), *nbr = (int*)(a + onbr);
        int *fc1 = (int*)(a + ofc1), *fc2 = (int*)(a + ofc2), *qc = (int*)(a + oqc);
        for (int gI = 0; gI < 14; gI++) geo_[gI] = (T*)(a + ogeo[gI]);
        t_ = (Q4<T>*)(a + ot); s_ = (T*)(a + os);
        P_ = (SolveParams<T>*)(a + oP); smax_ = (T*)(a + osmax); res2_ = (double*)(a + ores); flags_ = (int*)(a + oflag);
        tc_ = (Tile*)(a + otc); tf_ = (Tile*)(a + otf); cnt_ = (int*)(a + ocnt);
        tpart_ = (double*)(a + otp); srange_ = (int*)(a + osr);
        D_ = comp ? (Q4<T>*)(a + oD) : nullptr;
        Qlo_ = comp ? (Q4<T>*)(a + olo) : nullptr;
        m_.inc_off = incoff; m_.inc = inc; m_.nbr = nbr; m_.fc1 = fc1; m_.fc2 = fc2; m_.qcell = qc;
        m_.igeo = (const Q4<T>*)(a + oigeo);
        m_.g.nx = geo_[0]; m_.g.ny = geo_[1]; m_.g.area = geo_[2]; m_.g.c1dx = geo_[3]; m_.g.c1dy = geo_[4];
        m_.g.c2dx = geo_[5]; m_.g.c2dy = geo_[6]; m_.g.dxj = geo_[7]; m_.g.dyj = geo_[8]; m_.g.mx = geo_[9];
        m_.g.my = geo_[10]; m_.g.lx = geo_[11]; m_.g.ly = geo_[12]; m_.g.dist = geo_[13];
        m_.Ixx = ixx; m_.Iyy = iyy; m_.Ixy = ixy; m_.vol = vol;
        m_.rvol = (T*)(a + orvol); m_.rdist = (T*)(a + ordist);
        m_.fval = fv ? (Q4<T>*)(a + ofval) : nullptr;
        FV2D_B(cudaMemsetAsync(arena_, 0, bytes_, stream_));
        FV2D_B(cudaStreamSynchronize(stream_));
        cells_.reset(Nc_);
        faces_.reset(Fc_);
        incs_.reset(Ic_);
        recs_.assign(S_, Rec());
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev);
        compute_grids();
        return FV2D_OK;
    }

    int add(const fv2d_mesh_desc* d, const fv2d_case* cs, int* sid_out) override {
        HostMesh hm;
        int rc = build_mesh(d, cs, hm, err_);
        if (rc) return rc;
        rc = add_mesh(hm, cs, sid_out);
        // the uploads read hm's image, which goes with hm
        const cudaError_t e = cudaStreamSynchronize(stream_);
        if (!rc && e != cudaSuccess) { err_ = cudaGetErrorString(e); return FV2D_ERR_CUDA; }
        return rc;
    }

    // Upload image of one mesh: every per-solve array in arena format with solve-local ids, in one
    // page-locked block, so an admission is a few asynchronous copies plus an id-shift kernel.
    struct MeshImage {
        long long n = 0, m = 0, k = 0;
        char* pin = nullptr;
        size_t o_off = 0, o_inc = 0, o_nbr = 0, o_fc1 = 0, o_fc2 = 0, o_qc = 0, o_ixx = 0, o_iyy = 0, o_ixy = 0,
               o_vol = 0, o_igeo = 0, o_geo[14] = {};
        std::vector<int> n2o;
        ~MeshImage() { if (pin) cudaFreeHost(pin); }
    };

    int mesh_image(const HostMesh& hm, std::shared_ptr<MeshImage>& out) {
        auto& slot = hm.batch_image[sizeof(T) == 4 ? 1 : 0];
        if (slot) { out = std::static_pointer_cast<MeshImage>(slot); return FV2D_OK; }
        DeviceLayout L;
        build_layout(hm, L);
        auto im = std::make_shared<MeshImage>();
        im->n = hm.nc; im->m = hm.nf; im->k = L.ninc;
        size_t off = 0;
        auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 63) & ~size_t(63); return o; };
        const size_t n = (size_t)im->n, m = (size_t)im->m, k = (size_t)im->k;
        im->o_off = take(4 * (n + 1)); im->o_inc = take(4 * k); im->o_nbr = take(4 * k);
        im->o_fc1 = take(4 * m); im->o_fc2 = take(4 * m); im->o_qc = take(4 * m);
        im->o_ixx = take(8 * n); im->o_iyy = take(8 * n); im->o_ixy = take(8 * n);
        im->o_vol = take(sizeof(T) * n); im->o_igeo = take(sizeof(T) * 4 * k);
        for (int gI = 0; gI < 14; gI++) im->o_geo[gI] = take(sizeof(T) * m);
        FV2D_B(cudaMallocHost(&im->pin, off));
        auto cp = [&](size_t o, const void* src, size_t bytes) { std::memcpy(im->pin + o, src, bytes); };
        auto cpT = [&](size_t o, const std::vector<double>& src) {
            T* d = (T*)(im->pin + o);
            for (size_t i = 0; i < src.size(); i++) d[i] = (T)src[i];
        };
        cp(im->o_off, L.inc_off.data(), 4 * (n + 1)); cp(im->o_inc, L.inc.data(), 4 * k);
        cp(im->o_nbr, L.nbr.data(), 4 * k); cp(im->o_fc1, L.fc1.data(), 4 * m); cp(im->o_fc2, L.fc2.data(), 4 * m);
        cp(im->o_qc, L.qcell.data(), 4 * m);
        cp(im->o_ixx, L.Ixx.data(), 8 * n); cp(im->o_iyy, L.Iyy.data(), 8 * n); cp(im->o_ixy, L.Ixy.data(), 8 * n);
        cpT(im->o_vol, L.vol); cpT(im->o_igeo, L.igeo);
        for (int gI = 0; gI < 14; gI++) cpT(im->o_geo[gI], L.fgeo[gI]);
        im->n2o = hm.cell_new2old;
        slot = im;
        out = im;
        return FV2D_OK;
    }

    int add_mesh(const HostMesh& hm, const fv2d_case* cs, int* sid_out) override {
        if (hm.bc1 != cs->bc1 || hm.bc2 != cs->bc2) { err_ = "mesh was built with other BC codes than this case"; return FV2D_ERR_ARG; }
        int sid = -1;
        for (int i = 0; i < S_; i++) if (!recs_[i].active) { sid = i; break; }
        if (sid < 0) { err_ = "batch is full (max solves)"; return FV2D_ERR_NOMEM; }
        std::shared_ptr<MeshImage> im;
        int rc = mesh_image(hm, im);
        if (rc) return rc;
        Rec r;
        r.n = im->n; r.m = im->m; r.k = im->k;
        if (!cells_.alloc(r.n + 1, &r.c0)) { err_ = "batch cell capacity exhausted"; return FV2D_ERR_NOMEM; }
        if (!faces_.alloc(r.m, &r.f0)) { cells_.release(r.c0, r.n + 1); err_ = "batch face capacity exhausted"; return FV2D_ERR_NOMEM; }
        if (!incs_.alloc(r.k, &r.i0)) {
            cells_.release(r.c0, r.n + 1); faces_.release(r.f0, r.m);
            err_ = "batch incidence capacity exhausted"; return FV2D_ERR_NOMEM;
        }
        // asynchronous copies from the page-locked image (it outlives them: it is freed only with
        // the mesh, and a solve's mesh stays alive while it is admitted or the caller synchronises)
        const size_t n = (size_t)r.n, m = (size_t)r.m, k = (size_t)r.k;
        const char* P = im->pin;
        auto up = [&](const void* dst, size_t o, size_t bytes) {
            return cudaMemcpyAsync(const_cast<void*>(dst), P + o, bytes, cudaMemcpyHostToDevice, stream_);
        };
        FV2D_B(up(m_.inc_off + r.c0, im->o_off, 4 * (n + 1)));
        FV2D_B(up(m_.inc + r.i0, im->o_inc, 4 * k));
        FV2D_B(up(m_.nbr + r.i0, im->o_nbr, 4 * k));
        FV2D_B(up(m_.fc1 + r.f0, im->o_fc1, 4 * m));
        FV2D_B(up(m_.fc2 + r.f0, im->o_fc2, 4 * m));
        FV2D_B(up(m_.qcell + r.f0, im->o_qc, 4 * m));
        FV2D_B(up(m_.Ixx + r.c0, im->o_ixx, 8 * n));
        FV2D_B(up(m_.Iyy + r.c0, im->o_iyy, 8 * n));
        FV2D_B(up(m_.Ixy + r.c0, im->o_ixy, 8 * n));
        FV2D_B(up(m_.vol + r.c0, im->o_vol, sizeof(T) * n));
        FV2D_B(up(m_.igeo + r.i0, im->o_igeo, sizeof(T) * 4 * k));
        for (int gI = 0; gI < 14; gI++) FV2D_B(up(geo_[gI] + r.f0, im->o_geo[gI], sizeof(T) * m));
        {   // geometry reciprocals of the solve's ranges
            const long long mx = std::max<long long>(r.n, r.m);
            const int gr = (int)std::min<long long>((mx + 255) / 256, 4LL * sms_);
            k_reciprocals<T><<<gr, 256, 0, stream_>>>((int)r.m, geo_[13] + r.f0, (T*)m_.rdist + r.f0, (int)r.n,
                                                    m_.vol + r.c0, (T*)m_.rvol + r.c0);
            FV2D_B(cudaGetLastError());
        }
        // solve-local ids -> arena ids, on the device
        {
            const long long mx = std::max<long long>({r.n + 1, r.k, r.m});
            const int gr = (int)std::min<long long>((mx + 255) / 256, 4LL * sms_);
            k_shift_ids<int><<<gr, 256, 0, stream_>>>((int*)m_.inc_off + r.c0, (int)(r.n + 1), (int)r.i0, (int*)m_.inc + r.i0,
                                                (int*)m_.nbr + r.i0, (int)r.k, (int*)m_.fc1 + r.f0, (int*)m_.fc2 + r.f0,
                                                (int*)m_.qcell + r.f0, (int)r.m, (int)r.f0, (int)r.c0);
            FV2D_B(cudaGetLastError());
        }
        // parameters and the uniform freestream state (main.cpp:75-118)
        SolveParams<T> p{};
        const double gm1 = cs->gamma - 1, Cp = cs->R * cs->gamma / (cs->gamma - 1), kc = (cs->mu * Cp) / cs->Pr;
        const double E = (cs->P / (cs->gamma - 1)) + 0.5 * cs->rho * (cs->u * cs->u + cs->v * cs->v);
        p.k.gamma = (T)cs->gamma; p.k.gm1 = (T)gm1; p.k.R = (T)cs->R; p.k.mu = (T)cs->mu; p.k.k = (T)kc;
        p.k.q_inf[0] = (T)cs->rho; p.k.q_inf[1] = (T)(cs->rho * cs->u); p.k.q_inf[2] = (T)(cs->rho * cs->v); p.k.q_inf[3] = (T)E;
        p.k.rho_inf = (T)cs->rho; p.k.u_inf = (T)cs->u; p.k.v_inf = (T)cs->v; p.k.P_inf = (T)cs->P;
        p.k.two_cfl = (T)(2 * cs->cfl);
        p.k.vn0 = (T)std::sqrt(cs->v * cs->v + cs->u * cs->u);
        p.k.c0 = (T)std::sqrt(cs->gamma * (cs->P / cs->rho));
        p.k.roe = cs->flux_solver == FV2D_ROE;
        p.order2 = cs->order == 2; p.ns = cs->eqn == FV2D_NS; p.squeeze = cs->limiter == FV2D_LIM_SQUEEZE;
        p.global_dt = cs->time_type == FV2D_DT_GLOBAL; p.fresh = 1; p.init_prims = 1;
        pin_params_[sid] = p;   // a slot is rewritten only after its solve was removed (synchronised)
        FV2D_B(cudaMemcpyAsync(P_ + sid, pin_params_ + sid, sizeof(p), cudaMemcpyHostToDevice, stream_));
        // as the single-solve upload: hi = the state rounded to T, lo = the rounded remainder
        const double qd[4] = {cs->rho, cs->rho * cs->u, cs->rho * cs->v, E};
        Q4<T> hi1, lo1;
        for (int j = 0; j < 4; j++) { hi1.p[j] = (T)qd[j]; lo1.p[j] = (T)(qd[j] - (double)hi1.p[j]); }
        {
            const int gr = (int)std::min<long long>((r.n + 255) / 256, 4LL * sms_);
            k_fill_q<T><<<gr, 256, 0, stream_>>>(Q_[0] + r.c0, Qlo_ ? Qlo_ + r.c0 : nullptr, (int)r.n, hi1, lo1);
            FV2D_B(cudaGetLastError());
        }
        FV2D_B(cudaMemsetAsync(flags_ + sid, 0, 4, stream_));
        FV2D_B(cudaMemsetAsync(smax_ + sid, 0, sizeof(T), stream_));
        k_spectral_init<T><<<(int)((n + 255) / 256), 256, 0, stream_>>>((int)n, m_.inc_off + r.c0, m_.inc, m_.g.area,
                                                                         S_arr_ + r.c0, smax_ + sid, p.k);
        FV2D_B(cudaGetLastError());
        r.n2o = im->n2o;
        r.image = im;   // keeps the copies' source alive until the solve is removed
        r.active = true;
        recs_[sid] = std::move(r);
        *sid_out = sid;
        tiles_dirty_ = true;   // rebuilt once before the next step, after every admission of a round
        return FV2D_OK;
    }

    int remove(int sid) override {
        if (sid < 0 || sid >= S_ || !recs_[sid].active) { err_ = "no such solve"; return FV2D_ERR_ARG; }
        FV2D_B(cudaStreamSynchronize(stream_));
        Rec& r = recs_[sid];
        cells_.release(r.c0, r.n + 1);
        faces_.release(r.f0, r.m);
        incs_.release(r.i0, r.k);
        r = Rec();
        tiles_dirty_ = true;
        return FV2D_OK;
    }

    int step(int iterations) override {
        if (iterations < 0) { err_ = "negative iteration count"; return FV2D_ERR_ARG; }
        if (tiles_dirty_) {
            const int rc = rebuild_tiles();
            if (rc) return rc;
        }
        if (n_ctiles_ == 0) return FV2D_OK;
        for (int it = 0; it < iterations; it++) {
            if (timing_) {
                int rc = launch_iteration();
                if (rc) return rc;
            } else {
                if (!graph_) {
                    cudaGraph_t g;
                    FV2D_B(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
                    int rc = launch_iteration();
                    cudaError_t e = cudaStreamEndCapture(stream_, &g);
                    if (rc) return rc;
                    if (e != cudaSuccess) { err_ = std::string("graph capture: ") + cudaGetErrorString(e); return FV2D_ERR_CUDA; }
                    e = cudaGraphInstantiate(&graph_, g, 0);
                    cudaGraphDestroy(g);
                    if (e != cudaSuccess) { graph_ = nullptr; err_ = std::string("graph instantiate: ") + cudaGetErrorString(e); return FV2D_ERR_CUDA; }
                }
                FV2D_B(cudaGraphLaunch(graph_, stream_));
            }
            for (auto& r : recs_) if (r.active) r.iterations++;
        }
        return FV2D_OK;
    }

    int norms(int* sids, double* out, int* iters, int max, int* n) override {
        int rc = synchronize();
        std::vector<double> h(4 * (size_t)S_);
        FV2D_B(cudaMemcpy(h.data(), res2_, 32 * (size_t)S_, cudaMemcpyDeviceToHost));
        int k = 0;
        for (int s = 0; s < S_ && k < max; s++) {
            if (!recs_[s].active) continue;
            sids[k] = s;
            if (iters) iters[k] = recs_[s].iterations;
            for (int j = 0; j < 4; j++) out[4 * k + j] = std::sqrt(h[4 * s + j]);
            k++;
        }
        *n = k;
        return rc;
    }

    int get_state(int sid, double* q) override {
        if (sid < 0 || sid >= S_ || !recs_[sid].active) { err_ = "no such solve"; return FV2D_ERR_ARG; }
        const Rec& r = recs_[sid];
        std::vector<Q4<T>> h(r.n), lo(Qlo_ ? r.n : 0);
        FV2D_B(cudaStreamSynchronize(stream_));
        FV2D_B(cudaMemcpy(h.data(), Q_[0] + r.c0, sizeof(Q4<T>) * r.n, cudaMemcpyDeviceToHost));
        if (Qlo_) FV2D_B(cudaMemcpy(lo.data(), Qlo_ + r.c0, sizeof(Q4<T>) * r.n, cudaMemcpyDeviceToHost));
        for (long long c = 0; c < r.n; c++) {
            const int o = r.n2o[c];
            for (int j = 0; j < 4; j++)   // FP64: the value itself (adding 0.0 would turn -0 into +0)
                q[(size_t)j * r.n + o] = Qlo_ ? (double)h[c].p[j] + (double)lo[c].p[j] : (double)h[c].p[j];
        }
        int f = 0;
        FV2D_B(cudaMemcpy(&f, flags_ + sid, 4, cudaMemcpyDeviceToHost));
        if (f) { err_ = "non-physical state (rho <= 0, E <= 0 or NaN) in this solve"; return FV2D_ERR_STATE; }
        return FV2D_OK;
    }

    int synchronize() override {
        FV2D_B(cudaStreamSynchronize(stream_));
        return FV2D_OK;
    }

    int set_tuning(const BatchTuning& t) override {
        if (t.block < 64 || t.block > kBatchMaxBlock || (t.block & 31)) {
            err_ = "block must be a multiple of 32 in [64, " + std::to_string(kBatchMaxBlock) + "]";
            return FV2D_ERR_ARG;
        }
        for (int b = 0; b < 3; b++) if (t.tile_mult[b] < 1 || t.tile_mult[b] > 64) { err_ = "tile multiple out of range"; return FV2D_ERR_ARG; }
        FV2D_B(cudaStreamSynchronize(stream_));
        tune_ = t;
        compute_grids();
        if (graph_) { cudaGraphExecDestroy(graph_); graph_ = nullptr; }
        return rebuild_tiles();
    }
    BatchTuning tuning() const override { return tune_; }

    int usage(long long* o) override {
        long long act = 0;
        for (auto& r : recs_) act += r.active;
        o[0] = cells_.used(); o[1] = cells_.cap(); o[2] = faces_.used(); o[3] = faces_.cap();
        o[4] = incs_.used(); o[5] = incs_.cap(); o[6] = act; o[7] = (long long)bytes_;
        return FV2D_OK;
    }

    int set_timing(int enable) override {
        timing_ = enable != 0;
        for (int i = 0; i < 3; i++) { ms_[i] = 0; launches_[i] = 0; }
        return FV2D_OK;
    }
    int kernel_times(double* ms, int* launches) override {
        FV2D_B(cudaStreamSynchronize(stream_));
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
    void* stream() override { return (void*)stream_; }

private:
    int bucket(long long cells) const {
        return cells < tune_.bucket_edges[0] ? 0 : cells < tune_.bucket_edges[1] ? 1 : 2;
    }

    int rebuild_tiles() {
        tiles_dirty_ = false;
        std::vector<Tile> tc, tf;
        std::vector<int> sr(2 * (size_t)S_, 0);   // per solve slot: first cell tile, cell tile count
        for (int s = 0; s < S_; s++) {
            const Rec& r = recs_[s];
            sr[2 * s] = (int)tc.size();
            if (!r.active) continue;
            const long long tile = (long long)tune_.block * tune_.tile_mult[bucket(r.n)];
            for (long long c = 0; c < r.n; c += tile) tc.push_back(Tile{s, (int)(r.c0 + c), (int)std::min(tile, r.n - c), 0});
            for (long long f = 0; f < r.m; f += tile) tf.push_back(Tile{s, (int)(r.f0 + f), (int)std::min(tile, r.m - f), 0});
            sr[2 * s + 1] = (int)tc.size() - sr[2 * s];
        }
        if ((int)tc.size() > tile_cap_ || (int)tf.size() > tile_cap_) { err_ = "tile list capacity exceeded"; return FV2D_ERR_NOMEM; }
        // asynchronous upload through a page-locked buffer; an event guards the buffer until the
        // previous upload has been read (the graph reads the device lists in stream order)
        const size_t bt = sizeof(Tile) * tc.size(), bf = sizeof(Tile) * tf.size(), bs = 4 * sr.size();
        const size_t need = bt + bf + bs + 64;
        FV2D_B(cudaEventSynchronize(tiles_free_));
        if (need > tile_pin_bytes_) {
            if (tile_pin_) cudaFreeHost(tile_pin_);
            tile_pin_ = nullptr;
            tile_pin_bytes_ = 0;
            FV2D_B(cudaMallocHost(&tile_pin_, 2 * need));
            tile_pin_bytes_ = 2 * need;
        }
        int* cnt = (int*)tile_pin_;
        cnt[0] = (int)tc.size();
        cnt[1] = (int)tf.size();
        char* tp = tile_pin_ + 64;
        if (bt) std::memcpy(tp, tc.data(), bt);
        if (bf) std::memcpy(tp + bt, tf.data(), bf);
        std::memcpy(tp + bt + bf, sr.data(), bs);
        if (bt) FV2D_B(cudaMemcpyAsync(tc_, tp, bt, cudaMemcpyHostToDevice, stream_));
        if (bf) FV2D_B(cudaMemcpyAsync(tf_, tp + bt, bf, cudaMemcpyHostToDevice, stream_));
        FV2D_B(cudaMemcpyAsync(srange_, tp + bt + bf, bs, cudaMemcpyHostToDevice, stream_));
        FV2D_B(cudaMemcpyAsync(cnt_, cnt, 2 * sizeof(int), cudaMemcpyHostToDevice, stream_));
        FV2D_B(cudaEventRecord(tiles_free_, stream_));
        n_ctiles_ = (int)tc.size();
        n_ftiles_ = (int)tf.size();
        if (tune_.full_grid) {   // grid sizes are baked into the captured graph
            compute_grids();
            if (graph_) { cudaGraphExecDestroy(graph_); graph_ = nullptr; }
        }
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

    int grid_for(const void* kernel) {
        int per = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, tune_.block, 0);
        return std::max(1, per) * sms_;
    }
    void compute_grids() {
        if (tune_.full_grid) {   // one block per tile: grids follow the tile counts
            gg_ = gu_[0] = gu_[1] = gu_[2] = std::max(1, n_ctiles_);
            gf_[0] = gf_[1] = std::max(1, n_ftiles_);
            return;
        }
        gg_ = grid_for((const void*)kb_gradient<T>);
        gf_[0] = grid_for((const void*)kb_face<T, false>);
        gf_[1] = grid_for((const void*)kb_face<T, true>);
        gu_[0] = grid_for((const void*)kb_update<T, 0>);
        gu_[1] = grid_for((const void*)kb_update<T, 1>);
        gu_[2] = grid_for((const void*)kb_update<T, 2>);
    }

    int launch_iteration() {
        const int B = tune_.block;
        const int* nct = cnt_;
        const int* nft = cnt_ + 1;
        for (int s = 0; s < 3; s++) {
            const int p = (s + 2) % 3;
            timed(0, [&] {
                kb_gradient<T><<<gg_, B, 0, stream_>>>(tc_, nct, m_, P_, Q_[s], Q_[p], G_[p], G_[s]);
            });
            timed(1, [&] {
                if (s == 2)
                    kb_face<T, true><<<gf_[1], B, 0, stream_>>>(tf_, nft, m_, P_, Q_[s], G_[s], t_, s_);
                else
                    kb_face<T, false><<<gf_[0], B, 0, stream_>>>(tf_, nft, m_, P_, Q_[s], G_[s], t_, s_);
            });
            if (s == 2) FV2D_B(cudaMemsetAsync(smax_, 0, sizeof(T) * S_, stream_));
            timed(2, [&] {
                if (s == 0)
                    kb_update<T, 0><<<gu_[0], B, 0, stream_>>>(tc_, nct, m_, P_, t_, s_, Q_[0], Q_[1], Q_[2], dt_, S_arr_, smax_, tpart_, flags_, D_, Qlo_);
                else if (s == 1)
                    kb_update<T, 1><<<gu_[1], B, 0, stream_>>>(tc_, nct, m_, P_, t_, s_, Q_[0], Q_[1], Q_[2], dt_, S_arr_, smax_, tpart_, flags_, D_, Qlo_);
                else
                    kb_update<T, 2><<<gu_[2], B, 0, stream_>>>(tc_, nct, m_, P_, t_, s_, Q_[0], Q_[1], Q_[2], dt_, S_arr_, smax_, tpart_, flags_, D_, Qlo_);
            });
            if (s == 2) kb_res_norm<T><<<S_, 256, 0, stream_>>>(srange_, tpart_, res2_);
            FV2D_B(cudaGetLastError());
        }
        return FV2D_OK;
    }
    struct Pending { int kid; cudaEvent_t a, b; };

    long long Nc_ = 0, Fc_ = 0, Ic_ = 0;
    int S_ = 0, sms_ = 1, tile_cap_ = 0, n_ctiles_ = 0, n_ftiles_ = 0;
    bool tiles_dirty_ = false;
    int gg_ = 1, gf_[2] = {1, 1}, gu_[3] = {1, 1, 1};
    BatchTuning tune_;
    cudaStream_t stream_ = nullptr;
    cudaGraphExec_t graph_ = nullptr;
    void* arena_ = nullptr;
    size_t bytes_ = 0;
    char* tile_pin_ = nullptr;                 // page-locked staging of the tile lists
    size_t tile_pin_bytes_ = 0;
    cudaEvent_t tiles_free_ = nullptr;         // the last tile upload has been read
    SolveParams<T>* pin_params_ = nullptr;     // page-locked source slot of each solve's parameters
    Q4<T>* Q_[3] = {nullptr, nullptr, nullptr};
    Q4<T>* G_[3] = {nullptr, nullptr, nullptr};
    T *dt_ = nullptr, *S_arr_ = nullptr, *s_ = nullptr, *smax_ = nullptr;
    T* geo_[14] = {nullptr};
    Q4<T>* t_ = nullptr;
    Q4<T>* D_ = nullptr;     // FP32 only: RK increment in delta form
    Q4<T>* Qlo_ = nullptr;   // FP32 only: compensation term of Qn
    SolveParams<T>* P_ = nullptr;
    double* res2_ = nullptr;
    double* tpart_ = nullptr;   // per cell tile: residual sums of squares of the last stage
    int* srange_ = nullptr;     // per solve slot: first cell tile and tile count
    int* flags_ = nullptr;
    Tile *tc_ = nullptr, *tf_ = nullptr;
    int* cnt_ = nullptr;
    DevMesh<T> m_{};
    RangeAlloc cells_, faces_, incs_;
    std::vector<Rec> recs_;
    bool timing_ = false;
    std::vector<Pending> pending_;
    std::vector<cudaEvent_t> free_events_;
    double ms_[3] = {0, 0, 0};
    int launches_[3] = {0, 0, 0};
};

#undef FV2D_B

}  // namespace fv2d
