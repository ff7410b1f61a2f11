// fv2d_residual_noalloc: first-order residual on caller-provided device arrays, with the per-face
// scratch in a fixed static device array, so the call allocates no memory at all.
//
// Who needs it: a caller whose device memory is entirely owned by another allocator (a host
// application that reserves the GPU's memory up front in its own pool, so a cudaMalloc from this
// library would fail or fragment that pool), or a latency-critical thread that must not call
// cudaMalloc/cudaFree because they can synchronise the whole device.  Such a caller passes its
// inputs and outputs as device pointers it already owns; the only extra memory is the static array
// below, which lives with this library's device code on each GPU until the process exits.  With
// CUDA's lazy module loading (the default) that code and the array are placed on a device by the
// first call there, so that first call takes device memory and later calls take none: callers
// whose allocator reserves the GPU make one warm-up call per device before reserving, or set
// CUDA_MODULE_LOADING=EAGER.
//
// Built with -fmad=false, like the FP64 engine, so its arithmetic rounds like the rest of the FP64
// path.  The existing entry points and kernels are untouched.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "fv2d_gpu.h"
#include "fv2d_kernels.cuh"

namespace fv2d {
void set_global_error(const std::string& msg);   // fv2d_api.cu: the text fv2d_last_error(NULL) returns

namespace {

// Face scratch: the residual contribution (V*A - F*A) of every face, 4 doubles per face.
// FV2D_NOALLOC_MAX_FACES * 4 * 8 bytes = 8 MiB.
__device__ __align__(256) double g_noalloc_face_scratch[FV2D_NOALLOC_MAX_FACES * 4];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_addr[kMaxDevices] = {nullptr};

// One-time set-up per device, with that device current: the device address of the scratch
// array.  In host code the symbol's name is only a host-side stand-in, never a device address.
// The address is cached per device ordinal for the life of the process; it belongs to the
// device's primary context, so a device reset after the first call is not supported.
int scratch_address(double** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { set_global_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e)); return FV2D_ERR_NODEV; }
    if (dev < 0 || dev >= kMaxDevices) { set_global_error("device ordinal out of range"); return FV2D_ERR_NODEV; }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_face_scratch);
        if (e != cudaSuccess || !p) {
            set_global_error(std::string("cudaGetSymbolAddress(face scratch): ") + cudaGetErrorString(e));
            return FV2D_ERR_CUDA;
        }
        g_scratch_addr[dev] = (double*)p;
    }
    *out = g_scratch_addr[dev];
    return FV2D_OK;
}

// Face pass: first-order reconstruction (face states are the cell states), boundary ghosts,
// Rusanov flux (reconstruction.cpp:22-80, class_f.hpp:41-50, rusanov.cpp:20-36); writes the face's
// residual contribution (res.cpp:81-89) into the scratch.  First order carries no viscous flux
// (res.cpp:27-29), for EULER and NS alike.
__global__ void __launch_bounds__(256)
k_noalloc_face(int nf, const int* __restrict__ fc1, const int* __restrict__ fc2, const double* __restrict__ nx,
               const double* __restrict__ ny, const double* __restrict__ area, int nc, const double* __restrict__ q,
               double* __restrict__ scratch, Consts<double> k) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int c1 = fc1[f], c2 = fc2[f];
    const double fnx = nx[f], fny = ny[f], A = area[f];
    double L[4], Rq[4];
#pragma unroll
    for (int j = 0; j < 4; j++) L[j] = q[(size_t)j * nc + c1];
    double lrho, lu, lv, lP;
    prims(L, k, lrho, lu, lv, lP);
    const double lc = sqrt(k.gamma * (lP / lrho));
    if (c2 >= 0) {
#pragma unroll
        for (int j = 0; j < 4; j++) Rq[j] = q[(size_t)j * nc + c2];
    } else if (c2 == -1) {
#pragma unroll
        for (int j = 0; j < 4; j++) Rq[j] = k.q_inf[j];
    } else if (c2 == -2) {
        const double vn = lu * fnx + lv * fny;
        cons(lrho, lu - 2.0 * vn * fnx, lv - 2.0 * vn * fny, lP, k, Rq);
    } else if (c2 == -3) {
#pragma unroll
        for (int j = 0; j < 4; j++) Rq[j] = L[j];
    } else {
        cons(lrho, -lu, -lv, lP, k, Rq);
    }
    double rrho, ru, rv, rP;
    prims(Rq, k, rrho, ru, rv, rP);
    const double rc = sqrt(k.gamma * (rP / rrho));
    const double vn1 = lu * fnx + lv * fny;
    const double vn2 = ru * fnx + rv * fny;
    const double F1[4] = {lrho * vn1, lrho * lu * vn1 + lP * fnx, lrho * lv * vn1 + lP * fny, vn1 * (L[3] + lP)};
    const double F2[4] = {rrho * vn2, rrho * ru * vn2 + rP * fnx, rrho * rv * vn2 + rP * fny, vn2 * (Rq[3] + rP)};
    const double vna = (vn1 + vn2) / 2.0;
    const double ca = (lc + rc) / 2.0;
    const double lam = (fabs(vna) + ca) / 2.0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const double Fr = (F1[j] + F2[j]) / 2.0 - lam * (Rq[j] - L[j]);
        scratch[(size_t)4 * f + j] = (0.0 * A) - (Fr * A);
    }
}

// Cell pass: gather of the face contributions in the order the cell's face list gives (ascending
// face id reproduces the reference's scatter order, res.cpp:74-102), divided by the volume (:104-109).
__global__ void __launch_bounds__(256)
k_noalloc_gather(int nc, const int* __restrict__ off, const int* __restrict__ inc, const double* __restrict__ vol,
                 const double* __restrict__ scratch, double* __restrict__ r) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int i = off[c]; i < off[c + 1]; i++) {
        const int f = inc[i] >> 1;
        if (inc[i] & 1) {
#pragma unroll
            for (int j = 0; j < 4; j++) acc[j] -= scratch[(size_t)4 * f + j];
        } else {
#pragma unroll
            for (int j = 0; j < 4; j++) acc[j] += scratch[(size_t)4 * f + j];
        }
    }
    const double v = vol[c];
#pragma unroll
    for (int j = 0; j < 4; j++) r[(size_t)j * nc + c] = acc[j] / v;
}

}  // namespace
}  // namespace fv2d

extern "C" int fv2d_residual_noalloc(const fv2d_noalloc_mesh* m, const fv2d_case* cs, const double* q, double* r,
                                     void* stream) {
    using namespace fv2d;
    if (!m || !cs || !q || !r) { set_global_error("null argument"); return FV2D_ERR_ARG; }
    if (!m->face_cell1 || !m->face_cell2 || !m->face_nx || !m->face_ny || !m->face_area || !m->cell_face_offsets ||
        !m->cell_faces || !m->cell_vol) { set_global_error("null mesh array"); return FV2D_ERR_ARG; }
    if (m->num_cells <= 0 || m->num_faces <= 0) { set_global_error("empty mesh"); return FV2D_ERR_ARG; }
    if (m->num_faces > FV2D_NOALLOC_MAX_FACES) {
        set_global_error("num_faces " + std::to_string(m->num_faces) + " exceeds the static scratch limit of " +
                         std::to_string(FV2D_NOALLOC_MAX_FACES) + " faces; use fv2d_create/fv2d_stage instead");
        return FV2D_ERR_ARG;
    }
    if (!(cs->gamma > 1) || !(cs->rho > 0) || !(cs->P > 0)) { set_global_error("gamma > 1, rho > 0, P > 0 required"); return FV2D_ERR_CASE; }
    if (cs->flux_solver != FV2D_RUSANOV) { set_global_error("flux_solver must be RUSANOV"); return FV2D_ERR_CASE; }
    double* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    Consts<double> k{};
    k.gamma = cs->gamma;
    k.gm1 = cs->gamma - 1;
    k.R = cs->R;
    k.q_inf[0] = cs->rho;
    k.q_inf[1] = cs->rho * cs->u;
    k.q_inf[2] = cs->rho * cs->v;
    k.q_inf[3] = (cs->P / (cs->gamma - 1)) + 0.5 * cs->rho * (cs->u * cs->u + cs->v * cs->v);
    cudaStream_t st = (cudaStream_t)stream;
    k_noalloc_face<<<(m->num_faces + 255) / 256, 256, 0, st>>>(m->num_faces, m->face_cell1, m->face_cell2, m->face_nx,
                                                                m->face_ny, m->face_area, m->num_cells, q, scratch, k);
    k_noalloc_gather<<<(m->num_cells + 255) / 256, 256, 0, st>>>(m->num_cells, m->cell_face_offsets, m->cell_faces,
                                                                  m->cell_vol, scratch, r);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { set_global_error(std::string("launch: ") + cudaGetErrorString(e)); return FV2D_ERR_CUDA; }
    return FV2D_OK;
}

