// Device code of the FP32 engine: one fused kernel per SSP-RK3 stage over the tile layout of
// fv2d_tiles.h.  Each CTA takes tiles from a counter; per tile:
//   load    one thread issues bulk asynchronous copies (cp.async.bulk, the TMA engine) of the
//           tile's record block, csr block and core-cell states into shared memory on an mbarrier
//           (its halo list was copied, and its blocks prefetched into L2, during the previous
//           tile's last flux pass); every wait on an mbarrier is bounded and reports a timeout
//   gather  meanwhile, the states of the ring-1 and ring-2 cells (neighbours of the tile)
//   grad    LSQ gradient + squeeze limiter of every core and ring-1 cell (compute_gradient,
//           src/solver/cell_gradient.cpp:9-131; squeeze, src/solver/squeeze.cpp:9-155), each cell's
//           sums in ascending original face id; limited gradients stay in shared memory
//   flux    reconstruction + boundary ghosts (reconstruction.cpp:22-80), NS face terms (:86-164),
//           Rusanov flux (rusanov.cpp:20-36) of every face of a core cell; the face's contribution
//           V*A - F*A (res.cpp:81-89) overwrites its displacement row in shared memory
//   update  residual gather (res.cpp:74-109), time step (ssp_rk3.cpp:24-47) and the SSP-RK3 stage
//           (ssp_rk3.cpp:50-77) of the core cells, in the compensated delta form of the FP32 path;
//           on the last stage, per-warp spectral maxima and residual sums, folded into the solve's
//           maximum and the tile's norm partials at the next tile's top
// A face shared by two tiles is evaluated by both, with the same inputs and the same code, so both
// get the same value; every per-cell sum runs in a fixed order, so results do not depend on the
// tile schedule, and a solve gives the same bits alone and in a batch (both run these kernels).
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "fv2d_kernels.cuh"
#include "fv2d_tiles.h"

namespace fv2d {

struct __align__(16) TParams {   // per solve
    Consts<float> k;
    int order2, ns, squeeze, global_dt;
    int fresh, init_prims, pad0, pad1;
};
static_assert(sizeof(TParams) % 16 == 0, "TParams is copied in 16-byte pieces");

struct TArgs {
    const TileDesc* tiles;
    const int* ntiles;
    int* counter;              // [3] next tile of each stage kernel (kernel s zeroes stage s+1's)
    TParams* P;
    const uint32_t* rec;
    const uint16_t* csr;
    const int* halo;
    const int* qcell;
    Q4<float>* Q[3];           // stage inputs: Qn, Q1, Q2
    Q4<float>* G[3];           // limited gradient of each stage input (x, y per cell)
    Q4<float>* D;              // RK increment (delta form)
    Q4<float>* Qlo;            // compensation term of Qn
    Q4<float>* R;              // residual (null: not kept)
    float *dt, *S;
    const float *vol, *rvol;
    const float4* lsq;         // per cell: the LSQ inverse-moment terms (Ixx, Iyy, Ixy) rounded to FP32, 0
    float* smax;               // [solves] max spectral sum (GLOBAL dt; zeroed by the second stage)
    int nsmax;                 // entries of smax
    int* flags;                // [solves] non-physical state seen
    double* tpart;             // [tiles][4] residual sums of squares of the last stage (null: none)
    int* err;                  // bit 1: an mbarrier wait timed out; bit 2: a tile descriptor out of range
    int store_r;               // keep R on stages 0 and 1 too
};

// Shared-memory plan of one CTA (bytes; every region 16-byte aligned).
constexpr int kSmRecWords = 5 * kTileRecs + 3 * kTileGeo;
constexpr int kSmRec = 4 * kSmRecWords;
constexpr int kSmCsr = ((2 * kTileCsr + 15) / 16) * 16;
constexpr int kSmHalo = 4 * kTileCells;
constexpr int kSmCq = 16 * kTileCells;
constexpr int kSmCg = 32 * kTileGrad;
constexpr int kSmTotal = kSmRec + kSmCsr + kSmHalo + kSmCq + kSmCg;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t mb, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mb), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t mb, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
}
// Bounded wait for the mbarrier phase with the given parity: false after ~2^22 polls (each poll
// suspends the thread for a while, so this is far longer than any copy takes).
__device__ __forceinline__ bool mbar_wait(uint32_t mb, uint32_t parity) {
    for (int i = 0; i < (1 << 22); i++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mb), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}
// Bulk copy global -> shared (16-byte aligned addresses, size a multiple of 16), completing on mb.
__device__ __forceinline__ void tma_load(void* dst, const void* src, uint32_t bytes, uint32_t mb) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(mb)
                 : "memory");
}

__device__ __forceinline__ float fw(uint32_t w) { return __uint_as_float(w); }

// Asynchronous copy of a 16-byte aligned object (a tile descriptor, a solve's parameters) to shared
// memory; complete after cp.async.wait_all.
template <class T>
__device__ __forceinline__ void copy_async(T* dst, const T* src) {
    static_assert(sizeof(T) % 16 == 0, "16-byte pieces");
#pragma unroll
    for (int i = 0; i < (int)(sizeof(T) / 16); i++)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst) + 16 * i),
                     "l"(reinterpret_cast<const char*>(src) + 16 * i)
                     : "memory");
}


// Primitives of a conservative state; returns 1/rho for later quotients.
__device__ __forceinline__ void tprims(const float p[4], const Consts<float>& k, float& rho, float& u, float& v,
                                       float& P, float& y) {
    rho = p[0];
    y = 1.0f / rho;
    u = p[1] * y;
    v = p[2] * y;
    P = (p[3] - 0.5f * rho * (u * u + v * v)) * k.gm1;
}

template <int STAGE>
__global__ void __launch_bounds__(kTileCore, 3) k_tstage(TArgs a) {
    extern __shared__ __align__(128) unsigned char sm[];
    uint32_t* srec = reinterpret_cast<uint32_t*>(sm);
    uint16_t* scsr = reinterpret_cast<uint16_t*>(sm + kSmRec);
    int* shalo = reinterpret_cast<int*>(sm + kSmRec + kSmCsr);
    Q4<float>* cq = reinterpret_cast<Q4<float>*>(sm + kSmRec + kSmCsr + kSmHalo);
    Q4<float>* cg = reinterpret_cast<Q4<float>*>(sm + kSmRec + kSmCsr + kSmHalo + kSmCq);
    __shared__ TileDesc td;
    __shared__ __align__(16) TileDesc tdn;   // the next tile this CTA takes
    __shared__ TParams tp, tpn;   // this tile's solve parameters, the next tile's
    __shared__ __align__(8) unsigned long long mbar, mbar_h;
    __shared__ int s_next, s_ctr[2];
    __shared__ float redf[kTileCore / 32];      // last stage: per-warp spectral maxima of a tile
    __shared__ float redw[4][kTileCore / 32];   // and per-warp residual sums of squares

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t mb = smem_u32(&mbar), mbh = smem_u32(&mbar_h);
    uint32_t parity = 0, parity_h = 0;
    const int ntiles = *a.ntiles;
    const Q4<float>* __restrict__ Qin = a.Q[STAGE];
    const Q4<float>* __restrict__ Qprev = a.Q[(STAGE + 2) % 3];
    const Q4<float>* __restrict__ Gprev = a.G[(STAGE + 2) % 3];
    Q4<float>* __restrict__ Gout = a.G[STAGE];

    // thread 0 takes each next tile while the current one is being processed: its index during
    // the halo gather (whose own loads cover the atomic's latency; a barrier waits for the
    // thread's outstanding accesses), its descriptor by an asynchronous copy to shared memory
    // issued in the gradient pass; in the last flux pass (the halo list is free by then) it checks
    // the descriptor and starts the copy of the next tile's halo list, so that the next tile's
    // ring states are gathered while its other blocks are copied.  The solve's parameters are
    // reloaded only when the solve changes.
    int next_t = 0, tp_sid = -1, tpn_sid = -1;
    // (last stage) a tile's per-warp spectral maxima and residual sums are folded by the last warp
    // at the top of the next tile, while its blocks are copied (or at the end): the tile's maximum
    // into its solve's by an atomic, the sums of squares over the warps in FP64, in warp order, into
    // the tile's partials (batches' norms).  No barrier waits for either.
    int red_t = -1, red_sid = 0;
    auto fold = [&]() {
        if (STAGE != 2 || red_t < 0 || warp != kTileCore / 32 - 1) return;
        if (a.tpart && lane < 4) {
            double sum = 0.0;
            for (int w = 0; w < kTileCore / 32; w++) sum += (double)redw[lane][w];
            a.tpart[4 * (size_t)red_t + lane] = sum;
        }
        if (lane == 0) {
            float bm = 0.f;
            for (int w = 0; w < kTileCore / 32; w++) bm = max2(bm, redf[w]);
            atomic_max_pos(a.smax + red_sid, bm);
        }
        red_t = -1;
    };
    // (thread 0) the next tile's fate in s_next: its index, -1 (none left) or -2 (an empty slot of
    // a removed solve, or a descriptor out of range: skipped); for a tile, the halo copy on mbar_h,
    // whose phase also publishes tdn to the threads that wait on it
    auto decide = [&]() {
        if (next_t >= ntiles) { s_next = -1; return; }
        const TileDesc& d = tdn;
        if (d.ncore == 0) { s_next = -2; return; }
        const bool ok = d.ncore > 0 && d.ncore <= kTileCore && d.ncore + d.n1 <= kTileGrad &&
                        d.ncore + d.n1 + d.n2 <= kTileCells && d.nr <= kTileRecs && d.ngeo <= kTileGeo &&
                        d.ncc >= 0 && d.ncc <= d.nint && d.nint <= d.nrc && d.nrc <= d.ngeo && d.ngeo <= d.nr && d.fpw >= 32 && d.fpw <= 1024 &&
                        (d.fpw & 31) == 0 && d.nrp >= d.nr && d.ngp >= d.ngeo &&
                        5 * d.nrp + 3 * d.ngp <= kSmRecWords && d.ncsr <= kTileCsr && d.noff <= d.ncsr &&
                        d.n1 + d.n2 <= d.nhalo && d.nhalo <= kTileCells && (d.nrp & 3) == 0 && (d.ngp & 3) == 0 &&
                        (d.ncsr & 7) == 0 && (d.nhalo & 3) == 0 && (d.rec & 3) == 0 && (d.csr & 7) == 0 && (d.halo & 3) == 0;
        if (!ok) { atomicOr(a.err, 4); s_next = -2; return; }
        // the earlier generic accesses of the halo list are complete (a barrier precedes every
        // call); order them before the async-proxy writes
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const uint32_t bhal = 4u * (uint32_t)d.nhalo;
        mbar_expect_tx(mbh, bhal);
        if (bhal) tma_load(shalo, a.halo + d.halo, bhal, mbh);
        {   // the tile's other blocks into L2 now, so that the copies at its top come from L2
            const uint32_t brec = 4u * (uint32_t)(5 * d.nrp + 3 * d.ngp), bcsr = 2u * (uint32_t)d.ncsr,
                           bq = 16u * (uint32_t)d.ncore;
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a.rec + d.rec), "r"(brec) : "memory");
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a.csr + d.csr), "r"(bcsr) : "memory");
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(Qin + d.c0), "r"(bq) : "memory");
        }
        s_next = next_t;
    };
    // for the next kernel in the stream: the next stage's tile counter and, in the second stage
    // (which does not read them), the GLOBAL-dt maxima that the last stage accumulates; stages run
    // in order, and a restart mid-iteration zeroes the counters on the host
    if (blockIdx.x == 0 && tid == 0) a.counter[(STAGE + 1) % 3] = 0;
    if (STAGE == 1)
        for (int i = blockIdx.x * blockDim.x + tid; i < a.nsmax; i += gridDim.x * blockDim.x) a.smax[i] = 0.f;
    if (tid == 0) {
        mbar_init(mb, 1);
        mbar_init(mbh, 1);
        next_t = atomicAdd(a.counter + STAGE, 1);
        if (next_t < ntiles) tdn = a.tiles[next_t];
        decide();
    }
    __syncthreads();
    for (;;) {
        const int t = s_next;
        if (t == -1) {
            fold();
            break;
        }
        if (t == -2) {
            __syncthreads();   // every thread has read s_next
            if (tid == 0) {
                next_t = atomicAdd(a.counter + STAGE, 1);
                if (next_t < ntiles) tdn = a.tiles[next_t];
                decide();
            }
            __syncthreads();
            continue;
        }
        if (tid == 0) {
            td = tdn;
            if (td.sid != tp_sid) {
                tp = td.sid == tpn_sid ? tpn : a.P[td.sid];
                tp_sid = td.sid;
            }
            // the previous tile's generic accesses of this shared memory are complete (barrier at
            // the end of the loop); order them before the async-proxy writes
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const TileDesc& d = td;
            const uint32_t brec = 4u * (uint32_t)(5 * d.nrp + 3 * d.ngp), bcsr = 2u * (uint32_t)d.ncsr,
                           bq = 16u * (uint32_t)d.ncore;
            mbar_expect_tx(mb, brec + bcsr + bq);
            tma_load(srec, a.rec + d.rec, brec, mb);
            tma_load(scsr, a.csr + d.csr, bcsr, mb);
            tma_load(cq, Qin + d.c0, bq, mb);
            // L2 prefetches (bulk, asynchronous) of the tile's rows that the gradient and update
            // passes read with plain loads later; rounded out to 16 bytes, inside the arena
            auto pf = [&](const void* p, size_t bytes) {
                const size_t lo = (size_t)p & ~(size_t)15, hi = ((size_t)p + bytes + 15) & ~(size_t)15;
                asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(lo), "r"((uint32_t)(hi - lo)) : "memory");
            };
            const size_t n = (size_t)d.ncore;
            if (tp.order2 && tp.squeeze) { pf(Qprev + d.c0, 16 * n); pf(Gprev + 2 * (size_t)d.c0, 32 * n); }
            if (tp.order2) pf(a.lsq + d.c0, 16 * n);
            pf(a.rvol + d.c0, 4 * n);
            if (STAGE == 0) { pf(a.vol + d.c0, 4 * n); pf(a.S + d.c0, 4 * n); }
            else { pf(a.Q[0] + d.c0, 16 * n); pf(a.D + d.c0, 16 * n); pf(a.dt + d.c0, 4 * n); }
            if (STAGE == 2) pf(a.Qlo + d.c0, 16 * n);
        }
        fold();   // the previous tile's last-stage reductions
        // ---- gather: the ring-1 and ring-2 states (after the halo copy; tdn is this tile's
        // descriptor until thread 0 requests the next one, after the barrier below), while the
        // other blocks are copied
        bool ok = mbar_wait(mbh, parity_h);
        parity_h ^= 1u;
        if (ok) {
            const int nh = tdn.n1 + tdn.n2, o = tdn.ncore, cb = tdn.cbase;
            for (int i = tid; i < nh; i += blockDim.x) cq[o + i] = Qin[cb + shalo[i]];
        }
        if (tid == 0) next_t = atomicAdd(a.counter + STAGE, 1);
        ok = mbar_wait(mb, parity) && ok;
        parity ^= 1u;
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicOr(a.err, 2);
            return;
        }

        const int ncore = td.ncore, n1 = td.n1, nrp = td.nrp, ngp = td.ngp;
        const int cbase = td.cbase, c0 = td.c0;
        const Consts<float>& k = tp.k;
        const bool order2 = tp.order2 != 0, ns = tp.ns != 0;
        const bool fresh = STAGE == 0 && tp.fresh != 0, init_prims = STAGE == 0 && tp.init_prims != 0;
        const bool squeeze = tp.squeeze != 0;
        const uint32_t* __restrict__ r_sl = srec;
        const float4* __restrict__ r_d = reinterpret_cast<const float4*>(srec + nrp);
        const float* __restrict__ r_nx = reinterpret_cast<const float*>(srec + 5 * nrp);
        const float* __restrict__ r_ny = reinterpret_cast<const float*>(srec + 5 * nrp + ngp);
        const float* __restrict__ r_A = reinterpret_cast<const float*>(srec + 5 * nrp + 2 * ngp);
        const uint16_t* __restrict__ c_off = scsr;
        const uint32_t* __restrict__ c_ent = reinterpret_cast<const uint32_t*>(scsr + td.noff);

        // ---- grad: the limited LSQ gradient of one core or ring-1 cell (local slot gI)
        auto grad_cell = [&](int gI) {
            {
                const int gid = gI < ncore ? c0 + gI : cbase + shalo[gI - ncore];
                const bool lim_prev = squeeze && !fresh;
                // requested first: used only after the loop over the cell's faces
                const float4 mom = a.lsq[gid];
                Q4<float> gpx, gpy;
                if (lim_prev) { gpx = Gprev[2 * (size_t)gid]; gpy = Gprev[2 * (size_t)gid + 1]; }
                const Q4<float> qc = cq[gI];
                // LSQ sums (Q(c2) - Q(c1)) * (dxj, dyj) over the cell's faces and, for the squeeze
                // limiter, the extremes over the neighbours of Q(n) - Q(c) (= the bounds Qmax - Q,
                // Qmin - Q of squeeze.cpp: rounding is monotone, so the extreme difference is the
                // difference of the extreme) and over the faces of gprev . (face centre - centre), the
                // previous face value's part that varies by face (its base Qprev - Q is added after
                // the loop, again exactly for the extremes)
                float sx[4] = {0.f, 0.f, 0.f, 0.f}, sy[4] = {0.f, 0.f, 0.f, 0.f};
                float dmin[4], dmax[4], tmin[4], tmax[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    dmin[j] = 0.f; dmax[j] = 0.f;
                    tmin[j] = 3.0e38f; tmax[j] = -3.0e38f;
                }
                // bit 15 of the end offset: the cell has a boundary face; the others' loop has no
                // boundary branches
                const uint32_t o1 = c_off[gI + 1];
                const int e0 = c_off[gI] & 0x7FFF, e1 = (int)(o1 & 0x7FFFu);
                auto face_loop = [&](auto interior) {
                    constexpr bool INTERIOR = decltype(interior)::value;
                    for (int e = e0; e < e1; e++) {
                        const uint32_t ent = c_ent[e];
                        const int r = (int)((ent & 0xFFFFu) >> 1), side = (int)(ent & 1u);
                        const int so = (int)(int16_t)(ent >> 16);   // the face's other cell (or BC code)
                        const float4 dd = r_d[r];
                        const float d1x = dd.x, d1y = dd.y, d2x = dd.z, d2y = dd.w;
                        float d[4];
                        if (INTERIOR || so >= 0) {
                            const Q4<float> qn = cq[so];
    #pragma unroll
                            for (int j = 0; j < 4; j++) {
                                d[j] = qn.p[j] - qc.p[j];
                                if (squeeze) { dmin[j] = fminf(dmin[j], d[j]); dmax[j] = fmaxf(dmax[j], d[j]); }
                            }
                        } else if (so == -1) {
    #pragma unroll
                            for (int j = 0; j < 4; j++) d[j] = k.q_inf[j] - qc.p[j];
                        } else if (so == -2 || so == -4) {
                            float rho, u, v, P, yr;
                            if (init_prims) { rho = k.rho_inf; u = k.u_inf; v = k.v_inf; P = k.P_inf; }
                            else if (so == -2) tprims(qc.p, k, rho, u, v, P, yr);
                            else {
                                const Q4<float> qq = Qin[cbase + a.qcell[td.rbase + r]];
                                tprims(qq.p, k, rho, u, v, P, yr);
                            }
                            float gq[4];
                            if (so == -2) {   // slip wall: the cell velocity reflected (cell_gradient.cpp:43-55)
                                const float fnx = r_nx[r], fny = r_ny[r];
                                const float vn = u * fnx + v * fny;
                                cons(rho, u - 2.0f * vn * fnx, v - 2.0f * vn * fny, P, k, gq);
                            } else {          // no-slip: cell `face id`'s state, velocity negated (:62-73)
                                cons(rho, -u, -v, P, k, gq);
                            }
    #pragma unroll
                            for (int j = 0; j < 4; j++) d[j] = gq[j] - qc.p[j];
                        } else {
    #pragma unroll
                            for (int j = 0; j < 4; j++) d[j] = 0.f;
                        }
                        // LSQ displacement c1 -> c2 (or ghost), times Q(c2) - Q(c1): for a c2-side cell the
                        // difference above is Q(c1) - Q(c2), so the displacement's sign is flipped instead
                        const float fx = side ? d2x - d1x : d1x - d2x, fy = side ? d2y - d1y : d1y - d2y;
                        const float ox = side ? d2x : d1x, oy = side ? d2y : d1y;   // face centre - this cell
    #pragma unroll
                        for (int j = 0; j < 4; j++) {
                            sx[j] += d[j] * fx;
                            sy[j] += d[j] * fy;
                            if (lim_prev) {
                                const float x = gpx.p[j] * ox + gpy.p[j] * oy;
                                tmin[j] = fminf(tmin[j], x);
                                tmax[j] = fmaxf(tmax[j], x);
                            }
                        }
                    }
                };
                // one loop per warp: the general one if any of its cells has a boundary face (a warp
                // running both would take the sum of the two)
                if (__any_sync(__activemask(), (o1 & 0x8000u) != 0)) face_loop(std::false_type{});
                else face_loop(std::true_type{});
                const float ixx = mom.x, iyy = mom.y, ixy = mom.z;
                Q4<float> gx, gy;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    gx.p[j] = sx[j] * iyy - sy[j] * ixy;
                    gy.p[j] = sy[j] * ixx - sx[j] * ixy;
                }
                if (squeeze) {
                    // squeeze (squeeze.cpp:68-141): phi = the smallest (bound - Q) / (face value - Q) over
                    // the faces whose previous face value leaves [Qmin, Qmax]; as x -> (bound - Q) / x is
                    // monotone on either side of zero, that is the quotient at the extreme t
                    Q4<float> qp;
                    if (lim_prev) qp = Qprev[gid];
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const float up = dmax[j], dn = dmin[j];
                        // t = (previous face value) - Q: its base plus the extremes above; -101 is the
                        // fresh face history's value
                        const float base = lim_prev ? qp.p[j] - qc.p[j] : -101.0f - qc.p[j];
                        const float thi = lim_prev ? base + tmax[j] : base, tlo = lim_prev ? base + tmin[j] : base;
                        float phi = 1.0f;
                        if (thi > up) phi = fminf(phi, up / thi);
                        if (tlo < dn) phi = fminf(phi, dn / tlo);
                        gx.p[j] *= phi;
                        gy.p[j] *= phi;
                    }
                }
                cg[2 * gI] = gx;
                cg[2 * gI + 1] = gy;
                if (gI < ncore) { Gout[2 * (size_t)gid] = gx; Gout[2 * (size_t)gid + 1] = gy; }
            }
        };

        // ---- flux of one face of a core cell (record r); V*A - F*A replaces its displacement row
        // and the spectral term its normal's x
            float4* w_t = reinterpret_cast<float4*>(srec + nrp);
            float* w_sp = reinterpret_cast<float*>(srec + 5 * nrp);
            const bool visc = ns && order2;   // first order never adds the viscous flux (res.cpp:27-29,50-53)
            // INTERIOR (a compile-time tag): the record joins two cells, so the boundary branches go
            // and both sides' reconstructions can be scheduled together
            auto flux_rec = [&](int r, auto interior) {
                constexpr bool INTERIOR = decltype(interior)::value;
                const uint32_t sl = r_sl[r];
                const int s1 = (int)(sl & 0xFFFFu), s2 = (int)(int16_t)(sl >> 16);
                const float4 dd = r_d[r];
                const float d1x = dd.x, d1y = dd.y, d2x = dd.z, d2y = dd.w;
                const float fnx = r_nx[r], fny = r_ny[r];
                const float mxf = -fny, myf = fnx;   // unit tangent p1 -> p2
                // face states; for NS also the face-average tangential derivative m.(grad Q1 + grad Q2)/2,
                // the difference Q2 - Q1 and c1's velocity, so the cell states and gradients die early
                float L[4], Rq[4], dm[4], dq[4];
                float cu = 0.f, cv = 0.f;
                {
                    const Q4<float> q1 = cq[s1];
                    Q4<float> g1x, g1y;
                    if (order2) { g1x = cg[2 * s1]; g1y = cg[2 * s1 + 1]; }
                    else {
#pragma unroll
                        for (int j = 0; j < 4; j++) { g1x.p[j] = 0.f; g1y.p[j] = 0.f; }
                    }
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        L[j] = q1.p[j] + g1x.p[j] * d1x + g1y.p[j] * d1y;
                        dm[j] = g1x.p[j] * mxf + g1y.p[j] * myf;
                        dq[j] = -q1.p[j];
                    }
                    if (!INTERIOR && visc && s2 == -4) {
                        if (init_prims) { cu = k.u_inf; cv = k.v_inf; }
                        else { const float yq = 1.0f / q1.p[0]; cu = q1.p[1] * yq; cv = q1.p[2] * yq; }
                    }
                }
                float lrho, lu, lv, lP, ly;
                tprims(L, k, lrho, lu, lv, lP, ly);
                if (INTERIOR || s2 >= 0) {
                    const Q4<float> q2 = cq[s2];
                    Q4<float> g2x, g2y;
                    if (order2) { g2x = cg[2 * s2]; g2y = cg[2 * s2 + 1]; }
                    else {
#pragma unroll
                        for (int j = 0; j < 4; j++) { g2x.p[j] = 0.f; g2y.p[j] = 0.f; }
                    }
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        Rq[j] = q2.p[j] + g2x.p[j] * d2x + g2y.p[j] * d2y;
                        dm[j] = 0.5f * (dm[j] + g2x.p[j] * mxf + g2y.p[j] * myf);
                        dq[j] += q2.p[j];
                    }
                } else if (s2 == -1) {
#pragma unroll
                    for (int j = 0; j < 4; j++) Rq[j] = k.q_inf[j];
                } else if (s2 == -2) {
                    const float vn = lu * fnx + lv * fny;
                    cons(lrho, lu - 2.0f * vn * fnx, lv - 2.0f * vn * fny, lP, k, Rq);
                } else if (s2 == -3) {
#pragma unroll
                    for (int j = 0; j < 4; j++) Rq[j] = L[j];
                } else {
                    cons(lrho, -lu, -lv, lP, k, Rq);
                }
                const float A = r_A[r];
                const float lc = sqrtf(k.gamma * lP * ly);
                float rrho, ru, rv, rP, ry;
                tprims(Rq, k, rrho, ru, rv, rP, ry);
                const float rc = sqrtf(k.gamma * rP * ry);
                const float vn1 = lu * fnx + lv * fny, vn2 = ru * fnx + rv * fny;
                const float vna = 0.5f * (vn1 + vn2), ca = 0.5f * (lc + rc);
                const float lam = 0.5f * (fabsf(vna) + ca);
                float Fr[4];
                {
                    const float F1[4] = {lrho * vn1, lrho * lu * vn1 + lP * fnx, lrho * lv * vn1 + lP * fny, vn1 * (L[3] + lP)};
                    const float F2[4] = {rrho * vn2, rrho * ru * vn2 + rP * fnx, rrho * rv * vn2 + rP * fny, vn2 * (Rq[3] + rP)};
#pragma unroll
                    for (int j = 0; j < 4; j++) Fr[j] = k.roe ? -101.0f : 0.5f * (F1[j] + F2[j]) - lam * (Rq[j] - L[j]);
                }
                float V[4] = {0.f, 0.f, 0.f, 0.f};
                if (visc) {
                    float Aq[4];
#pragma unroll
                    for (int j = 0; j < 4; j++) Aq[j] = 0.5f * (L[j] + Rq[j]);
                    float arho, au, av, aP, ya;
                    tprims(Aq, k, arho, au, av, aP, ya);
                    float ux = 0.f, uy = 0.f, vx = 0.f, vy = 0.f, Px = 0.f, Py = 0.f, rx = 0.f, rly = 0.f;
                    bool have = true;
                    if (INTERIOR || s2 >= 0) {
                        // l: unit vector c1 -> c2 (the LSQ displacement d1 - d2)
                        const float tx = d1x - d2x, ty = d1y - d2y;
                        const float yd = rsqrtf(tx * tx + ty * ty);
                        const float lxf = tx * yd, lyf = ty * yd;
                        float dQx[4], dQy[4];
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            const float dl = dq[j] * yd + dm[j];   // reconstruction.cpp:138-146: l for both terms
                            dQy[j] = dl * lyf;
                            dQx[j] = dl * lxf;
                        }
                        rx = dQx[0];
                        ux = dQx[1] - rx * au * ya;
                        vx = dQx[2] - rx * av * ya;
                        rly = dQy[0];
                        uy = dQy[1] - rly * au * ya;
                        vy = dQy[2] - rly * au * ya;   // reconstruction.cpp:155 uses u
                        Px = k.gm1 * (dQx[3] - 0.5f * rx * (au * au + av * av) - arho * (au * ux + av * vx));
                        Py = k.gm1 * (dQy[3] - 0.5f * rly * (au * au + av * av) - arho * (au * uy + av * vy));
                    } else if (s2 == -4) {
                        const float ydn = rsqrtf(d1x * d1x + d1y * d1y);
                        const float dudn = -cu * ydn, dvdn = -cv * ydn;
                        ux = dudn * fnx; uy = dudn * fny;
                        vx = dvdn * fnx; vy = dvdn * fny;
                    } else if (s2 == -2) {
                        have = false;   // SLIP_WALL with NS: tau and grad T stay zero (:104-106)
                    }
                    if (have) {
                        const float third = (ux + vy) * (1.0f / 3.0f);
                        const float txx = 2.0f * k.mu * (ux - third), txy = k.mu * (uy + vx), tyy = 2.0f * k.mu * (vy - third);
                        const float yden = 1.0f / (k.R * arho * arho);
                        const float dTx = (Px * arho - rx * aP) * yden, dTy = (Py * arho - rly * aP) * yden;
                        V[1] = txx * fnx + txy * fny;
                        V[2] = txy * fnx + tyy * fny;
                        V[3] = fnx * (au * txx + av * txy + k.k * dTx) + fny * (au * txy + av * tyy + k.k * dTy);
                    }
                }
                w_t[r] = make_float4((V[0] - Fr[0]) * A, (V[1] - Fr[1]) * A, (V[2] - Fr[2]) * A, (V[3] - Fr[3]) * A);
                if (STAGE == 2) w_sp[r] = k.roe ? (fabsf(k.vn0) + k.c0) * A : (fabsf(vna) + ca) * A;
            };

        // ---- schedule: core-cell gradients; then the ring-1 gradients on the first warps while the
        // other warps take the fluxes of faces between two core cells (they need core gradients
        // only), which the first warps join when done; then every remaining flux.  Fluxes go to
        // whole warps, td.fpw records at a time (the batch's faces-per-warp tuning), from shared
        // counters.
        if (tid == 0) { s_ctr[0] = 0; s_ctr[1] = 0; }
        if (order2) {
            if (tid == 0 && next_t < ntiles) copy_async(&tdn, a.tiles + next_t);
            // the history flags act only on an iteration's first stage (STAGE 0); the second stage's
            // kernel, which does not read them, clears them for the next iteration: once per solve
            // (the tile of its first cell), in a phase long enough to cover the stores
            if (STAGE == 1 && tid == 0 && c0 == cbase) { a.P[td.sid].fresh = 0; a.P[td.sid].init_prims = 0; }
            if (tid < ncore) grad_cell(tid);
            __syncthreads();
            if (tid == 0 && next_t < ntiles) {   // the next tile's solve parameters, if they change
                asm volatile("cp.async.wait_all;" ::: "memory");
                if (tdn.sid != tp_sid) { copy_async(&tpn, a.P + tdn.sid); tpn_sid = tdn.sid; }
            }
            // the first warps take the ring-1 gradients, then join the others on core-core fluxes
            if (tid < n1) grad_cell(ncore + tid);
            {
                const int fpw = td.fpw, ncc = td.ncc;
                for (;;) {
                    int base = 0;
                    if (lane == 0) base = atomicAdd(&s_ctr[0], fpw);
                    base = __shfl_sync(0xffffffffu, base, 0);
                    if (base >= ncc) break;
                    for (int r = base + lane; r < min(base + fpw, ncc); r += 32) flux_rec(r, std::true_type{});
                }
            }
        } else {
            if (tid == 0 && next_t < ntiles) copy_async(&tdn, a.tiles + next_t);
            if (STAGE == 1 && tid == 0 && c0 == cbase) { a.P[td.sid].fresh = 0; a.P[td.sid].init_prims = 0; }
        }
        __syncthreads();
        if (tid == 0) {   // the next tile: its descriptor checked, its halo list copied (free now)
            if (next_t < ntiles) asm volatile("cp.async.wait_all;" ::: "memory");
            decide();
        }
        {
            const int start = min(s_ctr[0], td.ncc), nrc = td.nrc, fpw = td.fpw, nint = td.nint;
            for (;;) {
                int base = 0;
                if (lane == 0) base = start + atomicAdd(&s_ctr[1], fpw);
                base = __shfl_sync(0xffffffffu, base, 0);
                if (base >= nrc) break;
                for (int r = base + lane; r < min(base + fpw, nrc); r += 32) {
                    if (r < nint) flux_rec(r, std::true_type{});
                    else flux_rec(r, std::false_type{});
                }
            }
        }
        __syncthreads();

        // ---- update: residual gather, time step, SSP-RK3 stage of the core cells
        float snext = 0.f;
        float r2[4] = {0.f, 0.f, 0.f, 0.f};
        if (tid < ncore) {
            const int c = tid, gid = c0 + c;
            const float4* tt = reinterpret_cast<const float4*>(srec + nrp);
            const float* sp = reinterpret_cast<const float*>(srec + 5 * nrp);
            // the stage's cell data, requested before the gather
            const float yv = a.rvol[gid];
            float dtc = 0.f, sc = 0.f, vc = 0.f;
            if (STAGE == 0) { vc = a.vol[gid]; if (!tp.global_dt) sc = a.S[gid]; }
            else dtc = a.dt[gid];
            Q4<float> qn, dprev, lo;
            if (STAGE == 0) qn = cq[c];
            else { qn = a.Q[0][gid]; dprev = a.D[gid]; }
            if (STAGE == 2) lo = a.Qlo[gid];
            float r4[4] = {0.f, 0.f, 0.f, 0.f};
            const int e0 = c_off[c] & 0x7FFF, e1 = c_off[c + 1] & 0x7FFF;
            for (int e = e0; e < e1; e++) {
                const uint32_t ent = c_ent[e];
                const int r = (int)((ent & 0xFFFFu) >> 1), side = (int)(ent & 1u);
                const float4 tv = tt[r];
                r4[0] += neg_if(tv.x, side);
                r4[1] += neg_if(tv.y, side);
                r4[2] += neg_if(tv.z, side);
                r4[3] += neg_if(tv.w, side);
                if (STAGE == 2) snext += sp[r];
            }
#pragma unroll
            for (int j = 0; j < 4; j++) r4[j] *= yv;
            if (a.R && (a.store_r || STAGE == 2)) { Q4<float> rr; for (int j = 0; j < 4; j++) rr.p[j] = r4[j]; a.R[gid] = rr; }
            if (STAGE == 0) {
                dtc = (k.two_cfl * vc) / (tp.global_dt ? a.smax[td.sid] : sc);
                a.dt[gid] = dtc;
            }
            Q4<float> out, dn;
            if (STAGE == 0) {
#pragma unroll
                for (int j = 0; j < 4; j++) { dn.p[j] = dtc * r4[j]; out.p[j] = qn.p[j] + dn.p[j]; }
                a.D[gid] = dn;
                a.Q[1][gid] = out;
            } else if (STAGE == 1) {
#pragma unroll
                for (int j = 0; j < 4; j++) { dn.p[j] = 0.25f * dprev.p[j] + 0.25f * dtc * r4[j]; out.p[j] = qn.p[j] + dn.p[j]; }
                a.D[gid] = dn;
                a.Q[2][gid] = out;
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const float inc = (2.0f / 3.0f) * dprev.p[j] + (2.0f / 3.0f) * dtc * r4[j];
                    float s, err;
                    two_sum(qn.p[j], lo.p[j] + inc, s, err);
                    out.p[j] = s;
                    lo.p[j] = err;
                }
                a.Q[0][gid] = out;
                a.Qlo[gid] = lo;
                a.S[gid] = snext;
#pragma unroll
                for (int j = 0; j < 4; j++) r2[j] = r4[j] * r4[j];
            }
            if (!positive(out.p[0]) || !positive(out.p[3])) atomicOr(a.flags + td.sid, 1);
        }
        if (STAGE == 2) {
            // per warp: the spectral maximum (GLOBAL dt of the next iteration) and, for a batch, the
            // residual sums of squares (its per-solve norms), squares and sums in FP32; the warps'
            // values are folded at the next tile's top (fold: fixed order, FP64 across warps; GB300's
            // FP64 unit is narrow, so only four lanes of one warp do FP64 arithmetic)
            float m = snext;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = max2(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (a.tpart) {
#pragma unroll
                for (int j = 0; j < 4; j++)
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) r2[j] += __shfl_xor_sync(0xffffffffu, r2[j], o);
            }
            if (lane == 0) {
                redf[warp] = m;
#pragma unroll
                for (int j = 0; j < 4; j++) redw[j][warp] = r2[j];
            }
            red_t = t;
            red_sid = td.sid;
        }
        __syncthreads();
    }
}

// Initial spectral sums of a solve's tiles (the initial Vn_avg, c_avg of every face,
// class_q.hpp:61-62) in each cell's csr order, and their maximum.
__global__ void __launch_bounds__(kTileCore) k_tspec_init(const TileDesc* __restrict__ tiles, int first, int count,
                                                        const uint32_t* __restrict__ rec, const uint16_t* __restrict__ csr,
                                                        const TParams* __restrict__ P, float* __restrict__ S,
                                                        float* __restrict__ smax) {
    __shared__ float red[kTileCore / 32];
    for (int t = first + blockIdx.x; t < first + count; t += gridDim.x) {
        const TileDesc d = tiles[t];
        const Consts<float>& k = P[d.sid].k;
        float s = 0.f;
        if ((int)threadIdx.x < d.ncore) {
            const uint16_t* off = csr + d.csr;
            const uint16_t* ent = off + d.noff;
            const float* A = reinterpret_cast<const float*>(rec + d.rec + 5 * (size_t)d.nrp + 2 * (size_t)d.ngp);
            for (int e = off[threadIdx.x] & 0x7FFF; e < (off[threadIdx.x + 1] & 0x7FFF); e++) s += (fabsf(k.vn0) + k.c0) * A[ent[2 * e] >> 1];
            S[d.c0 + threadIdx.x] = s;
        }
        float m = s;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = max2(m, __shfl_xor_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
        __syncthreads();
        if (threadIdx.x == 0) {
            float bm = 0.f;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) bm = max2(bm, red[w]);
            atomic_max_pos(smax + d.sid, bm);
        }
        __syncthreads();
    }
}

// Per-solve residual sums of squares: solve s owns tiles [srange[2s], srange[2s] + srange[2s+1]);
// one block per solve slot adds their per-tile sums in a fixed order.
__global__ void __launch_bounds__(256) k_tres_norm(const int* __restrict__ srange, const double* __restrict__ tpart,
                                                   double* __restrict__ res2) {
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

}  // namespace fv2d
