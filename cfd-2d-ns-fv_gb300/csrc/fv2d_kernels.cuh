// Device kernels of the fv2d residual-and-update step, templated on the state precision T.
//
// One RK stage = three launches:
//   k_gradient  (one thread per cell)  LSQ gradient over the cell's faces + squeeze limiter
//   k_face      (one thread per face)  reconstruction, boundary ghosts, NS face terms, Rusanov
//                                      flux; writes the face's residual contribution
//   k_update    (one thread per cell)  gathers the face contributions in ascending original face
//                                      id, divides by the volume, applies the SSP-RK3 stage, and
//                                      (last stage) the spectral sums for the next time step
// Every per-cell sum visits the cell's faces in ascending ORIGINAL face id, the order in which
// the reference's face loops scatter into the cell, so with T = double and FMA contraction off
// (-fmad=false) the results are bit-identical to the reference; no atomics touch the state.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fv2d {

template <class T>
struct alignas(4 * sizeof(T)) Q4 {
    T p[4];
};

template <class T>
struct Consts {
    T gamma, gm1, R, mu, k;            // gm1 = gamma - 1, k = mu*Cp/Pr (class_flow.hpp:36-40)
    T q_inf[4];                        // freestream conservative state (class_flow.hpp:28-34)
    T rho_inf, u_inf, v_inf, P_inf;    // freestream primitives (initial Qbar primitives)
    T two_cfl;                         // 2*CFL
    T vn0, c0;                         // initial Vn_avg, c_avg (class_q.hpp:61-62)
    // flux_solver = ROE: the reference's res() calls no flux routine (res.cpp:62-69), so the
    // inviscid flux of every face is class_F::init's -101 (class_f.hpp:26-30) and Vn_avg, c_avg
    // (the time step's spectral terms) keep their initial values
    int roe;
};

// Face geometry, SoA, device order.
template <class T>
struct FaceGeo {
    const T *nx, *ny, *area, *c1dx, *c1dy, *c2dx, *c2dy, *dxj, *dyj, *mx, *my, *lx, *ly, *dist;
};

// Every mesh array a stage reads, device order (single solve) or arena order (batch).
template <class T>
struct DevMesh {
    const int *inc_off, *inc, *nbr, *fc1, *fc2, *qcell;
    const Q4<T>* igeo;   // per incidence (CSR order): dxj, dyj, offset of the face centre from the cell
    FaceGeo<T> g;
    const double *Ixx, *Iyy, *Ixy;
    const T* vol;
    // geometry-only reciprocals, computed once (k_reciprocals) with the same Recip<T>::of the kernels
    // would evaluate every stage: 1/|dist| per face (NS interior faces), 1/vol per cell
    const T *rdist, *rvol;
    // reconstructed face states of the last face pass, [2 nf]: 2f + side (the incidence code) holds
    // the state on cell c1's (side 0) or c2's (side 1) side of face f - exactly the stale face
    // values the next squeeze reads.  Null: the squeeze recomputes them from the previous stage's
    // state and limited gradient with the same expression.
    Q4<T>* fval;
};

template <class T>
__device__ __forceinline__ Q4<T> ldq(const Q4<T>* __restrict__ a, int i) {
    return a[i];
}

// Ordered comparison a < b.  For doubles it runs on the integer pipe: a non-NaN double's bit
// pattern, with -0 folded onto +0 and the magnitude bits of negatives inverted, orders exactly as
// IEEE '<' (equal values, +0 and -0 included, give equal keys), and the compare and select issue on
// the integer ALU pipe instead of taking a DSETP slot on GB300's narrow FP64 pipe.  (NaN inputs,
// which only arise in states already flagged as non-physical, may order differently.)
__device__ __forceinline__ long long order_key(double x) {
    long long b = __double_as_longlong(x);
    b = (b == (long long)0x8000000000000000ULL) ? 0LL : b;
    return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}
template <class T>
__device__ __forceinline__ bool less(T a, T b) { return a < b; }
template <>
__device__ __forceinline__ bool less<double>(double a, double b) { return order_key(a) < order_key(b); }

// std::min({a, b}) / std::max({a, b}) semantics (first argument wins ties)
template <class T>
__device__ __forceinline__ T min2(T a, T b) { return less(b, a) ? b : a; }
template <class T>
__device__ __forceinline__ T max2(T a, T b) { return less(a, b) ? b : a; }

// class_Q::updateflow for one state (class_q.hpp:131-141); T (temperature) is never read by the
// step and is not formed.
template <class T>
__device__ __forceinline__ void prims(const T p[4], const Consts<T>& k, T& rho, T& u, T& v, T& P) {
    rho = p[0];
    const T E = p[3];
    u = p[1] / rho;
    v = p[2] / rho;
    P = (E - (T(0.5) * rho * (u * u + v * v))) * k.gm1;
}

// Division sharing one reciprocal between several quotients with the same denominator.
// FP64: y = RN(1/b) (__drcp_rn), then two of Markstein's residual corrections
// (P. Markstein, "Computation of elementary functions on the IBM RISC System/6000 processor",
// IBM J. Res. Dev. 34(1), 1990): q0 = RN(a*y) is within 1.5 ulp of a/b, the first correction
// q1 = q0 + RN(a - b*q0)*y brings it within 1 ulp, and with that faithful q1 the residual
// a - b*q1 is exact and q2 = RN(q1 + (a - b*q1)*y) is the correctly rounded a/b.  Valid for
// normal operands whose quotient neither overflows nor underflows (all solver quantities); a zero
// numerator (checked on its bits, not with an FP64 compare) returns the exact signed zero a*y.
// Tested bit for bit against IEEE division.
// FP32 divides directly (the FP32 engine is built with approximate division).
template <class T>
struct Recip {
    static __device__ __forceinline__ T of(T b) { return T(1) / b; }
    static __device__ __forceinline__ T div(T a, T b, T) { return a / b; }
};
template <>
struct Recip<double> {
    static __device__ __forceinline__ double of(double b) { return __drcp_rn(b); }
    static __device__ __forceinline__ double div(double a, double b, double y) {
        const double q0 = a * y;
        if ((__double_as_longlong(a) << 1) == 0) return q0;   // a == +-0, tested on the integer pipe
        const double q1 = __fma_rn(__fma_rn(-b, q0, a), y, q0);
        return __fma_rn(__fma_rn(-b, q1, a), y, q1);
    }
};

// a/3.  FP64: one residual correction suffices for this divisor (two are needed in general).
// y = RN(1/3) = 1/3 (1 - 2^-54), so a*y is within half an ulp of a/3 and q0 = RN(a*y) is faithful;
// r = a - 3 q0 is then exact (an integer multiple of ulp(q0), below 3 ulp), and q0 + r*y is within
// 2^-53 ulp of a/3.  a/3 lies at least ulp/6 from every rounding midpoint (a - 3m, m a midpoint,
// is a non-zero multiple of ulp/2), so RN(q0 + r*y) is the correctly rounded a/3.  Checked against
// IEEE division on the host (tests/cpu_helpers/div3_check.cpp).
template <class T>
__device__ __forceinline__ T div3(T a) { return Recip<T>::div(a, T(3), T(1.0 / 3.0)); }
template <>
__device__ __forceinline__ double div3<double>(double a) {
    const double y = 1.0 / 3.0, q0 = a * y;
    if ((__double_as_longlong(a) << 1) == 0) return q0;   // a == +-0
    return __fma_rn(__fma_rn(-3.0, q0, a), y, q0);
}

// +0 - x, IEEE round to nearest, for a term (V A) that is identically +0 (V = +0, area A >= +0):
// -x, and +0 when x is a zero of either sign
__device__ __forceinline__ double zero_minus(double x) {
    const long long b = __double_as_longlong(x) ^ (long long)0x8000000000000000ULL;
    return (b << 1) == 0 ? 0.0 : __longlong_as_double(b);
}
__device__ __forceinline__ float zero_minus(float x) {
    const int b = __float_as_int(x) ^ (int)0x80000000u;
    return (b << 1) == 0 ? 0.0f : __int_as_float(b);
}

// prims() with the reciprocal of rho shared by u, v (and returned for P/rho)
template <class T>
__device__ __forceinline__ void prims_r(const T p[4], const Consts<T>& k, T& rho, T& u, T& v, T& P, T& y) {
    rho = p[0];
    const T E = p[3];
    y = Recip<T>::of(rho);
    u = Recip<T>::div(p[1], rho, y);
    v = Recip<T>::div(p[2], rho, y);
    P = (E - (T(0.5) * rho * (u * u + v * v))) * k.gm1;
}

// class_flow::updateQ (class_flow.hpp:28-34)
template <class T>
__device__ __forceinline__ void cons(T rho, T u, T v, T P, const Consts<T>& k, T q[4]) {
    q[0] = rho;
    q[1] = rho * u;
    q[2] = rho * v;
    q[3] = (P / k.gm1) + T(0.5) * rho * (u * u + v * v);
}

// ------------------------------------------------------------------------------------------
// Gradient + squeeze limiter.  compute_gradient (src/solver/cell_gradient.cpp:9-131) and
// squeeze (src/solver/squeeze.cpp:9-155), restated as one gather per cell.
// The squeeze compares against the face values of the PREVIOUS stage (res.cpp:40 runs before the
// reconstruction at :48); they are recomputed here from the previous stage's state and limited
// gradient with the reconstruction's own expression, or are the -101 sentinel the face states
// start with (class_q.hpp:73-76) on the first stage after initialisation.
// a[j] for a run-time j without indexing (which would put the array in local memory)
template <class T>
__device__ __forceinline__ T pick4(const T a[4], int j) {
    return j == 0 ? a[0] : j == 1 ? a[1] : j == 2 ? a[2] : a[3];
}

#ifndef FV2D_FP32_BLOCK
#define FV2D_FP32_BLOCK 128   // threads per block of the FP32 single-solve gradient and face kernels
#endif
#ifndef FV2D_FP64_BLOCK
#define FV2D_FP64_BLOCK 128   // threads per block of the FP64 gradient and face kernels
#endif

// Shared-memory staging of the warp-shared limiter quotients (FP64 single solve, see gradient_cell)
#ifndef FV2D_WARPQ_CAP
#define FV2D_WARPQ_CAP 256   // flagged checks per warp held at once; warps with more use the per-cell loop
#endif
template <int WARPS>
struct WarpQ {
    double qc[WARPS][4][32], mn[WARPS][4][32], mx[WARPS][4][32];   // each cell's state and bounds
    int b[WARPS][32];                                               // each cell's first incidence
    unsigned short list[WARPS][FV2D_WARPQ_CAP];                     // (lane << 6) | check bit
    double quo[WARPS][FV2D_WARPQ_CAP];                              // the checks' quotients
};

template <class T, bool SQUEEZE, bool WARPQ = false, int QWARPS = FV2D_FP64_BLOCK / 32>
__device__ __forceinline__ void gradient_cell(int c, const DevMesh<T>& m, const Q4<T>* __restrict__ Q,
                                              const Q4<T>* __restrict__ Qprev, const Q4<T>* __restrict__ Gprev,
                                              Q4<T>* __restrict__ Gout, const Consts<T>& k, int first_stage,
                                              int init_prims) {
    const int* __restrict__ inc_off = m.inc_off;
    const int* __restrict__ inc = m.inc;
    const int* __restrict__ nbr = m.nbr;
    const int* __restrict__ qcell = m.qcell;
    const FaceGeo<T>& g = m.g;
    const Q4<T> qc = ldq(Q, c);
    T sx[4] = {T(0), T(0), T(0), T(0)}, sy[4] = {T(0), T(0), T(0), T(0)};
    T qmin[4], qmax[4];
    if (SQUEEZE)
        for (int j = 0; j < 4; j++) { qmin[j] = T(100000000000.0); qmax[j] = T(-100000000000.0); }
    const int b = inc_off[c], e = inc_off[c + 1];
    // software-pipelined: the next incidence's record and neighbour state are requested before
    // the current one is processed (every cell has at least 3 faces, so entry b exists)
    int inc_n = inc[b], nb_n = nbr[b];
    Q4<T> ig_n = ldq(m.igeo, b), qn_n;
    if (nb_n >= 0) qn_n = ldq(Q, nb_n);
    for (int i = b; i < e; i++) {
        const int f = inc_n >> 1, side = inc_n & 1, nb = nb_n;
        const Q4<T> ig = ig_n, qn = qn_n;
        if (i + 1 < e) {
            inc_n = inc[i + 1];
            nb_n = nbr[i + 1];
            ig_n = ldq(m.igeo, i + 1);
            if (nb_n >= 0) qn_n = ldq(Q, nb_n);
        }
        T d[4];
        if (nb >= 0) {
            const T* q1 = side == 0 ? qc.p : qn.p;   // reference orientation: c2 - c1
            const T* q2 = side == 0 ? qn.p : qc.p;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                d[j] = q2[j] - q1[j];
                if (SQUEEZE) {
                    qmin[j] = min2(qmin[j], min2(q1[j], q2[j]));
                    qmax[j] = max2(qmax[j], max2(q1[j], q2[j]));
                }
            }
        } else {
            if (nb == -1) {
#pragma unroll
                for (int j = 0; j < 4; j++) d[j] = k.q_inf[j] - qc.p[j];
            } else if (nb == -2 || nb == -4) {
                T rho, u, v, P, yr;
                if (init_prims) { rho = k.rho_inf; u = k.u_inf; v = k.v_inf; P = k.P_inf; }
                else if (nb == -2) prims_r(qc.p, k, rho, u, v, P, yr);
                else { const Q4<T> qq = ldq(Q, qcell[f]); prims_r(qq.p, k, rho, u, v, P, yr); }
                T gq[4];
                if (nb == -2) {        // slip wall: reflect the cell velocity (cell_gradient.cpp:43-55)
                    const T fnx = g.nx[f], fny = g.ny[f];
                    const T vn = u * fnx + v * fny;
                    cons(rho, u - T(2.0) * vn * fnx, v - T(2.0) * vn * fny, P, k, gq);
                } else {               // no-slip: state of cell `face id`, velocity negated (:62-73)
                    cons(rho, -u, -v, P, k, gq);
                }
#pragma unroll
                for (int j = 0; j < 4; j++) d[j] = gq[j] - qc.p[j];
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++) d[j] = T(0);
            }
            if (SQUEEZE)
#pragma unroll
                for (int j = 0; j < 4; j++) { qmin[j] = min2(qmin[j], qc.p[j]); qmax[j] = max2(qmax[j], qc.p[j]); }
        }
        const T fx = ig.p[0], fy = ig.p[1];
#pragma unroll
        for (int j = 0; j < 4; j++) { sx[j] += d[j] * fx; sy[j] += d[j] * fy; }
    }
    const T ixx = (T)m.Ixx[c], iyy = (T)m.Iyy[c], ixy = (T)m.Ixy[c];
    Q4<T> gx, gy;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        gx.p[j] = (sx[j] * iyy - sy[j] * ixy);
        gy.p[j] = (sy[j] * ixx - sx[j] * ixy);
    }
    if (SQUEEZE) {
        T phi[4] = {T(1), T(1), T(1), T(1)};
        Q4<T> qp, gpx, gpy;
        const Q4<T>* __restrict__ fval = sizeof(T) == 8 ? m.fval : nullptr;   // FP64 engine only
        if (!first_stage && !fval) { qp = ldq(Qprev, c); gpx = ldq(Gprev, 2 * c); gpy = ldq(Gprev, 2 * c + 1); }
        if constexpr (sizeof(T) == 8) {
            // FP64: only a minority of the (incidence, component) checks bound the face value and
            // need a quotient, but a conditional IEEE division is if-converted (computed for every
            // check).  So one pass flags the checks that need one (bit 4*(incidence - i0) + component,
            // 16 incidences per word) and a second loop takes one flagged check per trip - one
            // division per trip, so a warp runs as many divisions as its busiest cell has flags -
            // in ascending bit order, so every min2 applies in the original sequence per component.
            // An unflagged check's factor 1 leaves phi unchanged bit for bit (phi <= 1).
            // WARPQ (FP64 single solve, stored face states): a warp's flagged checks are listed in
            // shared memory and spread over its 32 lanes, one quotient per lane per round, so the
            // warp runs ceil(flagged / 32) divisions instead of its busiest cell's count; each cell
            // then applies its own quotients in ascending bit order, as the loop below does.
            bool shared_done = false;
            if constexpr (WARPQ) {
                constexpr unsigned FULL = 0xffffffffu;
                // taken by the whole warp or by none of it (the shuffles below need all 32 lanes):
                // a converged full warp whose cells all have at most 16 faces, in a block no larger
                // than the one the shared staging is sized for (QWARPS warps)
                if (fval != nullptr && blockDim.x <= 32 * QWARPS && __activemask() == FULL &&
                    __all_sync(FULL, e - b <= 16)) {
                    unsigned long long mask = 0;
                    for (int i = b; i < e; i++) {
                        Q4<T> qf;
                        if (first_stage) {
#pragma unroll
                            for (int j = 0; j < 4; j++) qf.p[j] = T(-101);
                        } else {
                            qf = ldq(fval, inc[i]);
                        }
#pragma unroll
                        for (int j = 0; j < 4; j++)
                            if (less(qf.p[j], qmin[j]) || less(qmax[j], qf.p[j])) mask |= 1ull << (4 * (i - b) + j);
                    }
                    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
                    const int cnt = __popcll(mask);
                    int incl = cnt;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int v = __shfl_up_sync(FULL, incl, o);
                        if (lane >= o) incl += v;
                    }
                    const int total = __shfl_sync(FULL, incl, 31), excl = incl - cnt;
                    if (total <= FV2D_WARPQ_CAP) {
                        __shared__ WarpQ<QWARPS> sq;
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            sq.qc[w][j][lane] = qc.p[j];
                            sq.mn[w][j][lane] = qmin[j];
                            sq.mx[w][j][lane] = qmax[j];
                        }
                        sq.b[w][lane] = b;
                        {
                            unsigned long long mm = mask;
                            int pos = excl;
                            while (mm) {
                                const int bit = __ffsll((long long)mm) - 1;
                                mm &= mm - 1;
                                sq.list[w][pos++] = (unsigned short)((lane << 6) | bit);
                            }
                        }
                        __syncwarp();
                        for (int g = lane; g < total; g += 32) {
                            const int ent = sq.list[w][g], ow = ent >> 6, bit = ent & 63, j = bit & 3;
                            const T qf = first_stage ? T(-101)
                                                     : reinterpret_cast<const T*>(fval)[4 * (size_t)inc[sq.b[w][ow] + (bit >> 2)] + j];
                            const T qcj = sq.qc[w][j][ow], mn = sq.mn[w][j][ow], mx = sq.mx[w][j][ow];
                            const T num = less(qf, mn) ? mn : mx;
                            sq.quo[w][g] = (num - qcj) / (qf - qcj);
                        }
                        __syncwarp();
                        {
                            unsigned long long mm = mask;
                            int pos = excl;
                            while (mm) {
                                const int bit = __ffsll((long long)mm) - 1;
                                mm &= mm - 1;
                                const int j = bit & 3;
                                const T ph = min2((T)sq.quo[w][pos++], pick4(phi, j));
#pragma unroll
                                for (int jj = 0; jj < 4; jj++) phi[jj] = jj == j ? ph : phi[jj];
                            }
                        }
                        __syncwarp();
                        shared_done = true;
                    }
                }
            }
            for (int i0 = b; i0 < (shared_done ? b : e); i0 += 16) {
                const int i1 = min(e, i0 + 16);
                unsigned long long mask = 0;
                for (int i = i0; i < i1; i++) {
                    Q4<T> qf;
                    if (first_stage) {
#pragma unroll
                        for (int j = 0; j < 4; j++) qf.p[j] = T(-101);
                    } else if (fval) {
                        qf = ldq(fval, inc[i]);
                    } else {
                        const Q4<T> ig = ldq(m.igeo, i);
#pragma unroll
                        for (int j = 0; j < 4; j++) qf.p[j] = qp.p[j] + gpx.p[j] * ig.p[2] + gpy.p[j] * ig.p[3];
                    }
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        if (less(qf.p[j], qmin[j]) || less(qmax[j], qf.p[j])) mask |= 1ull << (4 * (i - i0) + j);
                }
                while (mask) {
                    const int bit = __ffsll((long long)mask) - 1;
                    mask &= mask - 1;
                    const int j = bit & 3, i = i0 + (bit >> 2);
                    const T qcj = pick4(qc.p, j), mn = pick4(qmin, j), mx = pick4(qmax, j);
                    T qf;
                    if (first_stage) qf = T(-101);
                    else if (fval) qf = reinterpret_cast<const T*>(fval)[4 * (size_t)inc[i] + j];
                    else {
                        const Q4<T> ig = ldq(m.igeo, i);
                        qf = pick4(qp.p, j) + pick4(gpx.p, j) * ig.p[2] + pick4(gpy.p, j) * ig.p[3];
                    }
                    const T num = less(qf, mn) ? mn : mx;
                    const T ph = min2((num - qcj) / (qf - qcj), pick4(phi, j));
#pragma unroll
                    for (int jj = 0; jj < 4; jj++) phi[jj] = jj == j ? ph : phi[jj];
                }
            }
        } else {
            for (int i = b; i < e; i++) {
                const Q4<T> ig = ldq(m.igeo, i);
                const T dx = ig.p[2], dy = ig.p[3];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const T qf = first_stage ? T(-101) : qp.p[j] + gpx.p[j] * dx + gpy.p[j] * dy;
                    T ph = T(1);
                    if (less(qf, qmin[j])) ph = (qmin[j] - qc.p[j]) / (qf - qc.p[j]);
                    else if (less(qmax[j], qf)) ph = (qmax[j] - qc.p[j]) / (qf - qc.p[j]);
                    phi[j] = min2(ph, phi[j]);
                }
            }
        }
#pragma unroll
        for (int j = 0; j < 4; j++) { gx.p[j] = gx.p[j] * phi[j]; gy.p[j] = gy.p[j] * phi[j]; }
    }
    Gout[2 * c] = gx;
    Gout[2 * c + 1] = gy;
}

// Occupancy: the FP32 kernels are latency-bound gathers, so their register use is capped for more
// resident warps.  The FP64 kernels are FP64-pipe-bound; their block size and minimum resident
// blocks (register cap) set how many warps cover the pipe's latency.
#ifndef FV2D_FP64_GMINB
#define FV2D_FP64_GMINB 8   // 8 x 128 threads at 64 registers (spilling), 8 x 23 KB of shared memory:
                            // 4 % faster than half the warps at 128 registers
#endif
#ifndef FV2D_FP64_FMINB
#define FV2D_FP64_FMINB 4   // 4 x 128 threads at 116 registers
#endif
template <class T>
constexpr int kStageBlock = sizeof(T) == 4 ? FV2D_FP32_BLOCK : FV2D_FP64_BLOCK;   // gradient and face kernels

#ifndef FV2D_KG_MINB32
#define FV2D_KG_MINB32 8   // 8 x 128 threads at 61 registers, no spills: 3.5 % faster than 10 at 48
#endif
template <class T, bool SQUEEZE>
__global__ void __launch_bounds__(kStageBlock<T>, sizeof(T) == 4 ? FV2D_KG_MINB32 : FV2D_FP64_GMINB)
k_gradient(int nc, DevMesh<T> m, const Q4<T>* __restrict__ Q, const Q4<T>* __restrict__ Qprev,
           const Q4<T>* __restrict__ Gprev, Q4<T>* __restrict__ Gout, Consts<T> k, int first_stage, int init_prims) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    gradient_cell<T, SQUEEZE, sizeof(T) == 8>(c, m, Q, Qprev, Gprev, Gout, k, first_stage, init_prims);
}

// ------------------------------------------------------------------------------------------
// Face kernel: reconstruction + boundary ghosts (reconstruction.cpp:22-80), NS face terms
// (reconstruction.cpp:86-164, class_q.hpp:163-169, class_f.hpp:52-59), Rusanov flux
// (class_f.hpp:41-50, rusanov.cpp:20-36) and the face's residual contribution (res.cpp:81-89).
// Writes t = (V*A) - (F*A) per face and, on the last stage of an iteration, the spectral term
// (|Vn_avg| + c_avg)*A that the next time step sums (ssp_rk3.cpp:28-36).
template <class T, bool ORDER2, bool NS, bool LAST>
__device__ __forceinline__ void face_flux(int f, const DevMesh<T>& m, const Q4<T>* __restrict__ Q,
                                          const Q4<T>* __restrict__ G, Q4<T>* __restrict__ tout,
                                          T* __restrict__ sout, const Consts<T>& k, int init_prims) {
    const FaceGeo<T>& g = m.g;
    const int c1 = m.fc1[f], c2 = m.fc2[f];
    const T fnx = g.nx[f], fny = g.ny[f], A = g.area[f];
    const Q4<T> q1 = ldq(Q, c1);
    Q4<T> g1x, g1y;
    if (ORDER2) { g1x = ldq(G, 2 * c1); g1y = ldq(G, 2 * c1 + 1); }
    else {
#pragma unroll
        for (int j = 0; j < 4; j++) { g1x.p[j] = T(0); g1y.p[j] = T(0); }
    }
    // the right cell's loads are issued now, beside the left cell's (a boundary face, c2 < 0,
    // loads cell c1's row instead and never uses it), so the two gathers overlap
    const int c2l = c2 >= 0 ? c2 : c1;
    const Q4<T> q2l = ldq(Q, c2l);
    Q4<T> g2xl, g2yl;
    if (ORDER2) { g2xl = ldq(G, 2 * c2l); g2yl = ldq(G, 2 * c2l + 1); }
    T L[4], Rq[4];
    {
        const T dx = g.c1dx[f], dy = g.c1dy[f];
#pragma unroll
        for (int j = 0; j < 4; j++) L[j] = q1.p[j] + g1x.p[j] * dx + g1y.p[j] * dy;
    }
    T lrho, lu, lv, lP, ly;
    prims_r(L, k, lrho, lu, lv, lP, ly);
    const T lc = sqrt(k.gamma * Recip<T>::div(lP, lrho, ly));
    Q4<T> q2, g2x, g2y;
    if (c2 >= 0) {
        q2 = q2l;
        if (ORDER2) { g2x = g2xl; g2y = g2yl; }
        else {
#pragma unroll
            for (int j = 0; j < 4; j++) { g2x.p[j] = T(0); g2y.p[j] = T(0); }
        }
        const T dx = g.c2dx[f], dy = g.c2dy[f];
#pragma unroll
        for (int j = 0; j < 4; j++) Rq[j] = q2.p[j] + g2x.p[j] * dx + g2y.p[j] * dy;
    } else if (c2 == -1) {
#pragma unroll
        for (int j = 0; j < 4; j++) Rq[j] = k.q_inf[j];
    } else if (c2 == -2) {
        const T vn = lu * fnx + lv * fny;
        cons(lrho, lu - T(2.0) * vn * fnx, lv - T(2.0) * vn * fny, lP, k, Rq);
    } else if (c2 == -3) {
#pragma unroll
        for (int j = 0; j < 4; j++) Rq[j] = L[j];
    } else {
        cons(lrho, -lu, -lv, lP, k, Rq);
    }
    if constexpr (sizeof(T) == 8) {
        if (m.fval) {   // the next squeeze's stale face values (BC faces: the c1 side only)
            Q4<T> lq, rq;
#pragma unroll
            for (int j = 0; j < 4; j++) { lq.p[j] = L[j]; rq.p[j] = Rq[j]; }
            m.fval[2 * f] = lq;
            if (c2 >= 0) m.fval[2 * f + 1] = rq;
        }
    }
    T rrho, ru, rv, rP, ry_;
    prims_r(Rq, k, rrho, ru, rv, rP, ry_);
    const T rc = sqrt(k.gamma * Recip<T>::div(rP, rrho, ry_));

    // Rusanov
    const T vn1 = lu * fnx + lv * fny;
    const T vn2 = ru * fnx + rv * fny;
    const T F1[4] = {lrho * vn1, lrho * lu * vn1 + lP * fnx, lrho * lv * vn1 + lP * fny, vn1 * (L[3] + lP)};
    const T F2[4] = {rrho * vn2, rrho * ru * vn2 + rP * fnx, rrho * rv * vn2 + rP * fny, vn2 * (Rq[3] + rP)};
    const T vna = (vn1 + vn2) / T(2);
    const T ca = (lc + rc) / T(2);
    const T lam = (fabs(vna) + ca) / T(2);
    T Fr[4];
#pragma unroll
    for (int j = 0; j < 4; j++) Fr[j] = k.roe ? T(-101) : (F1[j] + F2[j]) / T(2) - lam * (Rq[j] - L[j]);

    // viscous flux (first order never adds it: res.cpp:27-29,50-53)
    T V[4] = {T(0), T(0), T(0), T(0)};
    if (NS && ORDER2) {
        T Aq[4];
#pragma unroll
        for (int j = 0; j < 4; j++) Aq[j] = T(0.5) * (L[j] + Rq[j]);
        T arho, au, av, aP, ya;
        prims_r(Aq, k, arho, au, av, aP, ya);
        T ux = T(0), uy = T(0), vx = T(0), vy = T(0), Px = T(0), Py = T(0), rx = T(0), ry = T(0);
        bool have = true;
        if (c2 >= 0) {
            const T ad = fabs(g.dist[f]);
            const T yd = m.rdist[f];   // Recip<T>::of(ad), precomputed
            // unit tangent p1 -> p2 (readmesh.cpp:400-406) from the normal: mx = dx/|d| = -ny and
            // my = dy/|d| = nx, bit for bit (same |d| expression, sign-symmetric rounding)
            const T mxf = -fny, myf = fnx, lxf = g.lx[f], lyf = g.ly[f];
            T dQx[4], dQy[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const T dl = Recip<T>::div(q2.p[j] - q1.p[j], ad, yd);
                const T dm = T(0.5) * (g1x.p[j] * mxf + g1y.p[j] * myf + g2x.p[j] * mxf + g2y.p[j] * myf);
                dQy[j] = dl * lyf + dm * lyf;
                dQx[j] = dl * lxf + dm * lxf;
            }
            rx = dQx[0];
            ux = dQx[1] - Recip<T>::div(rx * au, arho, ya);
            vx = dQx[2] - Recip<T>::div(rx * av, arho, ya);
            ry = dQy[0];
            uy = dQy[1] - Recip<T>::div(ry * au, arho, ya);
            vy = dQy[2] - Recip<T>::div(ry * au, arho, ya);   // reconstruction.cpp:155 uses u
            Px = k.gm1 * (dQx[3] - T(0.5) * rx * (au * au + av * av) - arho * (au * ux + av * vx));
            Py = k.gm1 * (dQy[3] - T(0.5) * ry * (au * au + av * av) - arho * (au * uy + av * vy));
        } else if (c2 == -4) {
            const T d1x = g.c1dx[f], d1y = g.c1dy[f];
            const T dn = fabs(sqrt(d1x * d1x + d1y * d1y));
            T cu, cv;
            if (init_prims) { cu = k.u_inf; cv = k.v_inf; }
            else { cu = q1.p[1] / q1.p[0]; cv = q1.p[2] / q1.p[0]; }
            const T ydn = Recip<T>::of(dn);
            const T dudn = Recip<T>::div(-cu, dn, ydn), dvdn = Recip<T>::div(-cv, dn, ydn);
            ux = dudn * fnx; uy = dudn * fny;
            vx = dvdn * fnx; vy = dvdn * fny;
        } else if (c2 == -2) {
            have = false;   // SLIP_WALL with NS: tau and grad T keep their initial zeros (:104-106)
        }
        T txx, txy, tyy, dTx, dTy;
        if (have) {
            const T third = div3(ux + vy);
            txx = T(2) * k.mu * (ux - third);
            txy = k.mu * (uy + vx);
            tyy = T(2) * k.mu * (vy - third);
            const T den = k.R * arho * arho, yden = Recip<T>::of(den);
            dTx = Recip<T>::div(Px * arho - rx * aP, den, yden);
            dTy = Recip<T>::div(Py * arho - ry * aP, den, yden);
        } else {
            txx = T(0); txy = T(0); tyy = T(0); dTx = T(0); dTy = T(0);
        }
        V[0] = T(0);
        V[1] = txx * fnx + txy * fny;
        V[2] = txy * fnx + tyy * fny;
        V[3] = fnx * (au * txx + av * txy + k.k * dTx) + fny * (au * txy + av * tyy + k.k * dTy);
    }
    Q4<T> t;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        // (V*A) - (F*A); V[0] is always +0, and all of V is +0 for Euler and first order
        if (j == 0 || !(NS && ORDER2)) t.p[j] = zero_minus(Fr[j] * A);
        else t.p[j] = (V[j] * A) - (Fr[j] * A);
    }
    tout[f] = t;
    if (LAST) sout[f] = k.roe ? (fabs(k.vn0) + k.c0) * A : (fabs(vna) + ca) * A;
}

#ifndef FV2D_KF_MINB32
#define FV2D_KF_MINB32 10   // 10 x 128 threads at 48 registers (16 B spill): 11 % faster than 8 at 63
#endif
template <class T, bool ORDER2, bool NS, bool LAST>
__global__ void __launch_bounds__(kStageBlock<T>, sizeof(T) == 4 ? FV2D_KF_MINB32 : FV2D_FP64_FMINB)
k_face(int nf, DevMesh<T> m, const Q4<T>* __restrict__ Q, const Q4<T>* __restrict__ G, Q4<T>* __restrict__ tout,
       T* __restrict__ sout, Consts<T> k, int init_prims) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    face_flux<T, ORDER2, NS, LAST>(f, m, Q, G, tout, sout, k, init_prims);
}

// ------------------------------------------------------------------------------------------
// Spectral sums S_c = sum_f (|Vn_avg| + c_avg) A_f in ascending original face id
// (ssp_rk3.cpp:28-36).  s == nullptr: the initial Vn_avg, c_avg of every face (class_q.hpp:61-62).
template <class T>
__device__ __forceinline__ void atomic_max_pos(T* addr, T v);
template <>
__device__ __forceinline__ void atomic_max_pos<double>(double* addr, double v) {
    atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}
template <>
__device__ __forceinline__ void atomic_max_pos<float>(float* addr, float v) {
    atomicMax(reinterpret_cast<unsigned int*>(addr), __float_as_uint(v));
}

template <class T>
__device__ __forceinline__ T block_max(T v) {
    __shared__ T red[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max2(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < (int)(blockDim.x >> 5) ? red[lane] : T(0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = max2(v, __shfl_xor_sync(0xffffffffu, v, o));
    }
    return v;
}

template <class T>
__global__ void __launch_bounds__(256)
k_spectral_init(int nc, const int* __restrict__ inc_off, const int* __restrict__ inc, const T* __restrict__ area,
                T* __restrict__ S, T* __restrict__ smax, Consts<T> k) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    T s = T(0);
    if (c < nc) {
        for (int i = inc_off[c]; i < inc_off[c + 1]; i++) s += (fabs(k.vn0) + k.c0) * area[inc[i] >> 1];
        S[c] = s;
    }
    const T m = block_max(c < nc ? s : T(0));
    if (threadIdx.x == 0) atomic_max_pos(smax, m);
}

// ------------------------------------------------------------------------------------------
// Residual gather + SSP-RK3 stage (res.cpp:74-109, ssp_rk3.cpp:38-77).
// STAGE 0: dt from the spectral sums (GLOBAL: 2*CFL*vol/max S, LOCAL: 2*CFL*vol/S), Q1 = Qn+dt*R
// STAGE 1: Q2 = 0.75*Qn + 0.25*Q1 + 0.25*dt*R
// STAGE 2: Qn = 1/3*Qn + 2/3*Q2 + 2/3*dt*R, and the spectral sums for the next iteration.
// Non-physical results (rho <= 0, E <= 0, NaN) raise bit 0 of *flag; values are kept as computed.
// FP32 keeps the RK increments in delta form and the base state as a compensated pair
// (hi + lo, error-free TwoSum), so increments below half an ulp of the state are not lost:
//   D1 = dt R1,               Q1 = hi + D1
//   D2 = D1/4 + dt R2 / 4,    Q2 = hi + D2
//   (hi, lo) += 2/3 D2 + 2/3 dt R3
// which is the SSP-RK3 combination of ssp_rk3.cpp:50-77 rewritten about Qn.  Gradients and fluxes
// read the FP32 stage states (hi, Q1, Q2).  FP64 (D == nullptr) keeps the reference's expressions.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}

// Incidences whose loads the residual gather issues together: 4 for FP64 (4.6 % faster k_update);
// 1 for FP32, where the wider chunk's registers cost the batch kernel more than it gains.
template <class T>
constexpr int kUpdChunk = sizeof(T) == 8 ? 4 : 1;

// S_c = sum of the face spectral terms in CSR order, loads issued a chunk at a time
template <class T>
__device__ __forceinline__ T spectral_sum(const int* __restrict__ inc, const T* __restrict__ sface, int b, int e) {
    T s = T(0);
    constexpr int U = kUpdChunk<T>;
    for (int i0 = b; i0 < e; i0 += U) {
        T v[U];
#pragma unroll
        for (int u = 0; u < U; u++)
            if (i0 + u < e) v[u] = sface[inc[i0 + u] >> 1];
#pragma unroll
        for (int u = 0; u < U; u++)
            if (i0 + u < e) s += v[u];
    }
    return s;
}

// -x when s == 1, x when s == 0: a sign-bit flip on the integer pipe.  r - t == r + (-t) exactly in
// IEEE arithmetic (zeros included), so the residual gather adds the flipped contribution instead
// of branching between += and -= on the incidence's side (a warp's lanes disagree on it).
__device__ __forceinline__ double neg_if(double x, int s) {
    return __longlong_as_double(__double_as_longlong(x) ^ ((long long)s << 63));
}
__device__ __forceinline__ float neg_if(float x, int s) { return __int_as_float(__float_as_int(x) ^ (s << 31)); }

// x > 0 (false for NaN).  FP64 on the integer pipe: 0 < bits <= bits(+inf).
template <class T>
__device__ __forceinline__ bool positive(T x) { return x > T(0); }
template <>
__device__ __forceinline__ bool positive<double>(double x) {
    return (unsigned long long)__double_as_longlong(x) - 1ull < 0x7ff0000000000000ull;
}

template <class T, int STAGE>
__device__ __forceinline__ T update_cell(int c, const DevMesh<T>& m, const Q4<T>* __restrict__ tface,
                                         const T* __restrict__ sface, Q4<T>* __restrict__ Qn, Q4<T>* __restrict__ Q1,
                                         Q4<T>* __restrict__ Q2, T* __restrict__ dt, T* __restrict__ S, T smax,
                                         Q4<T>* __restrict__ Rout, int* __restrict__ flag, const Consts<T>& k,
                                         int global_dt, T r[4], Q4<T>* __restrict__ D, Q4<T>* __restrict__ Qlo) {
    const int* __restrict__ inc = m.inc;
    T snext = T(0);
#pragma unroll
    for (int j = 0; j < 4; j++) r[j] = T(0);
    const int b = m.inc_off[c], e = m.inc_off[c + 1];
    // chunks of kUpdChunk incidences: every record and face contribution of a chunk is requested
    // before the first is summed (more loads in flight per thread); the sums keep CSR order
    constexpr int U = kUpdChunk<T>;
    for (int i0 = b; i0 < e; i0 += U) {
        int iv[U];
        Q4<T> tv[U];
#pragma unroll
        for (int u = 0; u < U; u++)
            if (i0 + u < e) iv[u] = inc[i0 + u];
#pragma unroll
        for (int u = 0; u < U; u++)
            if (i0 + u < e) tv[u] = ldq(tface, iv[u] >> 1);
#pragma unroll
        for (int u = 0; u < U; u++) {
            if (i0 + u < e) {
#pragma unroll
                for (int j = 0; j < 4; j++) r[j] += neg_if(tv[u].p[j], iv[u] & 1);   // side 1: r -= t
            }
        }
    }
    const T vc = m.vol[c];
    const T yv = m.rvol[c];   // Recip<T>::of(vc), precomputed
#pragma unroll
    for (int j = 0; j < 4; j++) r[j] = Recip<T>::div(r[j], vc, yv);
    if (Rout) { Q4<T> rr; for (int j = 0; j < 4; j++) rr.p[j] = r[j]; Rout[c] = rr; }
    const Q4<T> qn = ldq(Qn, c);
    Q4<T> out;
    T dtc;
    if (STAGE == 0) {
        dtc = (k.two_cfl * vc) / (global_dt ? smax : S[c]);
        dt[c] = dtc;
    } else {
        dtc = dt[c];
    }
    if constexpr (sizeof(T) == 4) {
        if (D) {
            Q4<T> d;
            if (STAGE == 0) {
#pragma unroll
                for (int j = 0; j < 4; j++) { d.p[j] = dtc * r[j]; out.p[j] = qn.p[j] + d.p[j]; }
                D[c] = d;
                Q1[c] = out;
            } else if (STAGE == 1) {
                const Q4<T> d1 = ldq((const Q4<T>*)D, c);
#pragma unroll
                for (int j = 0; j < 4; j++) { d.p[j] = T(0.25) * d1.p[j] + T(0.25) * dtc * r[j]; out.p[j] = qn.p[j] + d.p[j]; }
                D[c] = d;
                Q2[c] = out;
            } else {
                const Q4<T> d2 = ldq((const Q4<T>*)D, c);
                Q4<T> lo = ldq((const Q4<T>*)Qlo, c);
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const T inc_j = T(2.0 / 3.0) * d2.p[j] + T(2.0 / 3.0) * dtc * r[j];
                    T s, err;
                    two_sum(qn.p[j], lo.p[j] + inc_j, s, err);
                    out.p[j] = s;
                    lo.p[j] = err;
                }
                Qn[c] = out;
                Qlo[c] = lo;
                snext = spectral_sum(inc, sface, b, e);
                S[c] = snext;
            }
            if (!positive(out.p[0]) || !positive(out.p[3])) atomicOr(flag, 1);
            return snext;
        }
    }
    if (STAGE == 0) {
#pragma unroll
        for (int j = 0; j < 4; j++) out.p[j] = qn.p[j] + dtc * r[j];
        Q1[c] = out;
    } else if (STAGE == 1) {
        const Q4<T> q1 = ldq(Q1, c);
#pragma unroll
        for (int j = 0; j < 4; j++) out.p[j] = T(0.75) * qn.p[j] + T(0.25) * q1.p[j] + T(0.25) * dtc * r[j];
        Q2[c] = out;
    } else {
        const Q4<T> q2 = ldq(Q2, c);
#pragma unroll
        for (int j = 0; j < 4; j++)
            out.p[j] = T(1.0 / 3.0) * qn.p[j] + T(2.0 / 3.0) * q2.p[j] + T(2.0 / 3.0) * dtc * r[j];
        Qn[c] = out;
        snext = spectral_sum(inc, sface, b, e);
        S[c] = snext;
    }
    if (!positive(out.p[0]) || !positive(out.p[3])) atomicOr(flag, 1);
    return snext;
}

#ifndef FV2D_UPD_BLOCK
#define FV2D_UPD_BLOCK 256   // threads per block of the single-solve update kernel
#endif
template <class T, int STAGE>
__global__ void __launch_bounds__(FV2D_UPD_BLOCK)
k_update(int nc, DevMesh<T> m, const Q4<T>* __restrict__ tface, const T* __restrict__ sface, Q4<T>* __restrict__ Qn,
         Q4<T>* __restrict__ Q1, Q4<T>* __restrict__ Q2, T* __restrict__ dt, T* __restrict__ S, T* __restrict__ smax,
         Q4<T>* __restrict__ Rout, int* __restrict__ flag, Consts<T> k, int global_dt, Q4<T>* __restrict__ D,
         Q4<T>* __restrict__ Qlo) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    T snext = T(0);
    if (c < nc) {
        T r[4];
        snext = update_cell<T, STAGE>(c, m, tface, sface, Qn, Q1, Q2, dt, S, (STAGE == 0 && global_dt) ? *smax : T(0),
                                      Rout, flag, k, global_dt, r, D, Qlo);
    }
    if (STAGE == 2) {
        const T mx = block_max(c < nc ? snext : T(0));
        if (threadIdx.x == 0) atomic_max_pos(smax, mx);
    }
}

// Geometry-only reciprocals of a mesh (or of one solve's ranges in a batch arena): rdist = 1/|dist|
// (dist may be null: no NS faces) and rvol = 1/vol, with the kernels' own Recip<T>::of.
template <class T>
__global__ void k_reciprocals(int nf, const T* __restrict__ dist, T* __restrict__ rdist, int nc,
                              const T* __restrict__ vol, T* __restrict__ rvol) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < max(nf, nc); i += gridDim.x * blockDim.x) {
        if (i < nf && dist) rdist[i] = Recip<T>::of(fabs(dist[i]));
        if (i < nc) rvol[i] = Recip<T>::of(vol[i]);
    }
}

// ------------------------------------------------------------------------------------------
// Host-format <-> device-format state (SoA double in file numbering <-> AoS T in device order).
template <class T>
__global__ void k_state_in(int nc, const int* __restrict__ new2old, const double* __restrict__ q, Q4<T>* __restrict__ Q,
                           Q4<T>* __restrict__ Qlo) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int o = new2old[c];
    Q4<T> v, lo;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const double x = q[(size_t)j * nc + o];
        v.p[j] = (T)x;
        lo.p[j] = (T)(x - (double)v.p[j]);
    }
    Q[c] = v;
    if (Qlo) Qlo[c] = lo;
}

template <class T>
__global__ void k_state_out(int nc, int ncomp, const int* __restrict__ new2old, const Q4<T>* __restrict__ Q,
                            double* __restrict__ q, const Q4<T>* __restrict__ Qlo) {
    // ncomp = 4 (state; plus its compensation term when Qlo is given) or 8 (gradient pairs)
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    const int o = new2old[c];
    const int per = ncomp / 4;
    for (int h = 0; h < per; h++) {
        const Q4<T> v = Q[(size_t)per * c + h];
        Q4<T> lo;
        if (Qlo) lo = Qlo[c];
#pragma unroll
        // FP64 (no compensation term): the value itself - adding 0.0 would turn -0 into +0
        for (int j = 0; j < 4; j++) q[(size_t)(4 * h + j) * nc + o] = Qlo ? (double)v.p[j] + (double)lo.p[j] : (double)v.p[j];
    }
}

template <class T>
__global__ void k_scalar_out(int nc, const int* __restrict__ new2old, const T* __restrict__ a, double* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    out[new2old[c]] = (double)a[c];
}

// Sum of squares of the residual per variable, FP64, deterministic two-level reduction.
template <class T>
__global__ void __launch_bounds__(256) k_res_norm_partial(int nc, const Q4<T>* __restrict__ R, double* __restrict__ part) {
    __shared__ double sh[4][256];
    double acc[4] = {0, 0, 0, 0};
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const Q4<T> r = R[c];
#pragma unroll
        for (int j = 0; j < 4; j++) acc[j] += (double)r.p[j] * (double)r.p[j];
    }
#pragma unroll
    for (int j = 0; j < 4; j++) sh[j][threadIdx.x] = acc[j];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
#pragma unroll
            for (int j = 0; j < 4; j++) sh[j][threadIdx.x] += sh[j][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0)
#pragma unroll
        for (int j = 0; j < 4; j++) part[4 * blockIdx.x + j] = sh[j][0];
}

}  // namespace fv2d
