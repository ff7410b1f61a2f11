// Solver engine for one precision: device arena, stage sequencing, CUDA-graph replay of whole
// iterations, per-kernel event timing and host<->device field transfers.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fv2d_hostcopy.h"
#include "fv2d_kernels.cuh"
#include "fv2d_solver.h"

namespace fv2d {

#define FV2D_CUDA(call)                                                                         \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            err_ = std::string(#call) + ": " + cudaGetErrorString(e_);                          \
            return e_ == cudaErrorMemoryAllocation ? FV2D_ERR_NOMEM : FV2D_ERR_CUDA;            \
        }                                                                                       \
    } while (0)

template <class T>
class SolverImpl : public Solver {
public:
    ~SolverImpl() override {
        if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
        for (auto& p : pending_) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
        for (auto e : free_events_) cudaEventDestroy(e);
        if (arena_) cudaFree(arena_);
        if (host_stage_) cudaFreeHost(host_stage_);
        for (cudaEvent_t e : copy_events_) cudaEventDestroy(e);
        if (stage_free_) cudaEventDestroy(stage_free_);
        if (stream_) cudaStreamDestroy(stream_);
    }

    int init(const fv2d_case& cs) override {
        cs_ = cs;
        const HostMesh& m = mesh_;
        DeviceLayout L;
        build_layout(m, L);
        nc_ = m.nc; nf_ = m.nf; ninc_ = L.ninc;
        order2_ = cs.order == 2;
        ns_ = cs.eqn == FV2D_NS;
        squeeze_ = cs.limiter == FV2D_LIM_SQUEEZE;
        global_dt_ = cs.time_type == FV2D_DT_GLOBAL;
        // constants, evaluated like main.cpp:77-79 / class_flow.hpp
        const double gm1 = cs.gamma - 1;
        const double Cp = cs.R * cs.gamma / (cs.gamma - 1);
        const double kcond = (cs.mu * Cp) / cs.Pr;
        const double E = (cs.P / (cs.gamma - 1)) + 0.5 * cs.rho * (cs.u * cs.u + cs.v * cs.v);
        k_.gamma = (T)cs.gamma; k_.gm1 = (T)gm1; k_.R = (T)cs.R; k_.mu = (T)cs.mu; k_.k = (T)kcond;
        k_.q_inf[0] = (T)cs.rho; k_.q_inf[1] = (T)(cs.rho * cs.u); k_.q_inf[2] = (T)(cs.rho * cs.v); k_.q_inf[3] = (T)E;
        k_.rho_inf = (T)cs.rho; k_.u_inf = (T)cs.u; k_.v_inf = (T)cs.v; k_.P_inf = (T)cs.P;
        k_.two_cfl = (T)(2 * cs.cfl);
        k_.vn0 = (T)std::sqrt(cs.v * cs.v + cs.u * cs.u);
        k_.c0 = (T)std::sqrt(cs.gamma * (cs.P / cs.rho));
        k_.roe = cs.flux_solver == FV2D_ROE;

        FV2D_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
        // ---- arena layout
        size_t off = 0;
        auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
        const size_t q4 = sizeof(Q4<T>);
        const int ngeo = ns_ ? 14 : 9;
        size_t o_q[3], o_g[3];
        for (int i = 0; i < 3; i++) o_q[i] = take(q4 * nc_);
        for (int i = 0; i < 3; i++) o_g[i] = take(2 * q4 * nc_);
        size_t o_r = take(q4 * nc_), o_dt = take(sizeof(T) * nc_), o_S = take(sizeof(T) * nc_);
        size_t o_vol = take(sizeof(T) * nc_), o_ixx = take(8 * nc_), o_iyy = take(8 * nc_), o_ixy = take(8 * nc_);
        size_t o_rvol = take(sizeof(T) * nc_), o_rdist = take(sizeof(T) * nf_);
        size_t o_incoff = take(4 * (nc_ + 1)), o_inc = take(4 * (size_t)ninc_), o_nbr = take(4 * (size_t)ninc_);
        size_t o_igeo = take(q4 * (size_t)ninc_);
        size_t o_fc1 = take(4 * (size_t)nf_), o_fc2 = take(4 * (size_t)nf_), o_qcell = take(4 * (size_t)nf_);
        size_t o_geo[14];
        for (int gI = 0; gI < 14; gI++) o_geo[gI] = gI < ngeo ? take(sizeof(T) * nf_) : 0;
        size_t o_t = take(q4 * nf_), o_s = take(sizeof(T) * nf_);
        size_t o_smax = take(64), o_flag = take(64);
        size_t o_n2o = take(4 * (size_t)nc_);
        // FP64 squeeze: the face pass stores its reconstructed states for the next limiter pass
        // (the FP32 engine, memory-bound, recomputes them instead)
        const bool store_fval = sizeof(T) == 8 && order2_ && squeeze_;
        size_t o_fval = store_fval ? take(2 * q4 * (size_t)nf_) : 0;
        size_t o_stage = take(8 * 8 * (size_t)nc_);
        nred_ = 304;
        size_t o_part = take(8 * 4 * (size_t)nred_);
        const bool comp = sizeof(T) == 4;   // FP32: delta-form increments + compensated base state
        size_t o_D = comp ? take(q4 * nc_) : 0, o_lo = comp ? take(q4 * nc_) : 0;
        arena_bytes_ = off;
        FV2D_CUDA(cudaMalloc(&arena_, arena_bytes_));
        char* a = (char*)arena_;
        for (int i = 0; i < 3; i++) { Q_[i] = (Q4<T>*)(a + o_q[i]); G_[i] = (Q4<T>*)(a + o_g[i]); }
        R_ = (Q4<T>*)(a + o_r); dt_ = (T*)(a + o_dt); S_ = (T*)(a + o_S); vol_ = (T*)(a + o_vol);
        Ixx_ = (double*)(a + o_ixx); Iyy_ = (double*)(a + o_iyy); Ixy_ = (double*)(a + o_ixy);
        inc_off_ = (int*)(a + o_incoff); inc_ = (int*)(a + o_inc); nbr_ = (int*)(a + o_nbr);
        fc1_ = (int*)(a + o_fc1); fc2_ = (int*)(a + o_fc2); qcell_ = (int*)(a + o_qcell);
        T* geo[14];
        for (int gI = 0; gI < 14; gI++) geo[gI] = gI < ngeo ? (T*)(a + o_geo[gI]) : nullptr;
        g_.nx = geo[0]; g_.ny = geo[1]; g_.area = geo[2]; g_.c1dx = geo[3]; g_.c1dy = geo[4];
        g_.c2dx = geo[5]; g_.c2dy = geo[6]; g_.dxj = geo[7]; g_.dyj = geo[8];
        g_.mx = geo[9]; g_.my = geo[10]; g_.lx = geo[11]; g_.ly = geo[12]; g_.dist = geo[13];
        t_ = (Q4<T>*)(a + o_t); s_ = (T*)(a + o_s);
        dm_.inc_off = inc_off_; dm_.inc = inc_; dm_.nbr = nbr_; dm_.fc1 = fc1_; dm_.fc2 = fc2_; dm_.qcell = qcell_;
        dm_.igeo = (const Q4<T>*)(a + o_igeo);
        dm_.g = g_; dm_.Ixx = Ixx_; dm_.Iyy = Iyy_; dm_.Ixy = Ixy_; dm_.vol = vol_;
        dm_.rvol = (T*)(a + o_rvol); dm_.rdist = (T*)(a + o_rdist);
        dm_.fval = store_fval ? (Q4<T>*)(a + o_fval) : nullptr;
        smax_ = (T*)(a + o_smax); flag_ = (int*)(a + o_flag);
        n2o_ = (int*)(a + o_n2o); dstage_ = (double*)(a + o_stage); part_ = (double*)(a + o_part);
        D_ = comp ? (Q4<T>*)(a + o_D) : nullptr;
        Qlo_ = comp ? (Q4<T>*)(a + o_lo) : nullptr;
        FV2D_CUDA(cudaMemsetAsync(arena_, 0, arena_bytes_, stream_));
        // ---- upload (one pinned staging buffer reused for every array)
        staging_bytes_ = std::max<size_t>({sizeof(T) * (size_t)nf_, 8 * (size_t)nc_ * 8, 4 * (size_t)ninc_,
                                           4 * (size_t)(nc_ + 1), 4 * (size_t)nf_});
        FV2D_CUDA(cudaMallocHost(&host_stage_, staging_bytes_));
        FV2D_CUDA(cudaEventCreateWithFlags(&stage_free_, cudaEventDisableTiming));
        auto put = [&](void* dst, const void* src, size_t bytes) -> int {
            std::memcpy(host_stage_, src, bytes);
            FV2D_CUDA(cudaMemcpyAsync(dst, host_stage_, bytes, cudaMemcpyHostToDevice, stream_));
            FV2D_CUDA(cudaStreamSynchronize(stream_));
            return FV2D_OK;
        };
        auto putT = [&](T* dst, const std::vector<double>& src) -> int {
            T* h = (T*)host_stage_;
            for (size_t i = 0; i < src.size(); i++) h[i] = (T)src[i];
            FV2D_CUDA(cudaMemcpyAsync(dst, host_stage_, sizeof(T) * src.size(), cudaMemcpyHostToDevice, stream_));
            FV2D_CUDA(cudaStreamSynchronize(stream_));
            return FV2D_OK;
        };
        int rc;
        if ((rc = put(inc_off_, L.inc_off.data(), 4 * (nc_ + 1)))) return rc;
        if ((rc = put(inc_, L.inc.data(), 4 * (size_t)ninc_))) return rc;
        if ((rc = put(nbr_, L.nbr.data(), 4 * (size_t)ninc_))) return rc;
        if ((rc = put(fc1_, L.fc1.data(), 4 * (size_t)nf_))) return rc;
        if ((rc = put(fc2_, L.fc2.data(), 4 * (size_t)nf_))) return rc;
        if ((rc = put(qcell_, L.qcell.data(), 4 * (size_t)nf_))) return rc;
        if ((rc = put(n2o_, m.cell_new2old.data(), 4 * (size_t)nc_))) return rc;
        if ((rc = put(Ixx_, L.Ixx.data(), 8 * (size_t)nc_))) return rc;
        if ((rc = put(Iyy_, L.Iyy.data(), 8 * (size_t)nc_))) return rc;
        if ((rc = put(Ixy_, L.Ixy.data(), 8 * (size_t)nc_))) return rc;
        if ((rc = putT(vol_, L.vol))) return rc;
        for (int gI = 0; gI < ngeo; gI++) if ((rc = putT(geo[gI], L.fgeo[gI]))) return rc;
        for (size_t i0 = 0; i0 < L.igeo.size(); i0 += staging_bytes_ / sizeof(T)) {   // staged in chunks
            const size_t n0 = std::min(L.igeo.size() - i0, staging_bytes_ / sizeof(T));
            std::vector<double> part(L.igeo.begin() + i0, L.igeo.begin() + i0 + n0);
            if ((rc = putT((T*)(a + o_igeo) + i0, part))) return rc;
        }
        {
            const int mx = std::max(nf_, nc_);
            k_reciprocals<T><<<(mx + 255) / 256, 256, 0, stream_>>>(nf_, g_.dist, (T*)dm_.rdist, nc_, vol_, (T*)dm_.rvol);
            FV2D_CUDA(cudaGetLastError());
        }
        return reset_freestream();
    }

    // Uniform freestream Qbar (class_q.hpp:50-94 + updateQ) and initial face histories.
    int reset_freestream() {
        std::vector<double> q(4 * (size_t)nc_);
        const double E = (cs_.P / (cs_.gamma - 1)) + 0.5 * cs_.rho * (cs_.u * cs_.u + cs_.v * cs_.v);
        const double qq[4] = {cs_.rho, cs_.rho * cs_.u, cs_.rho * cs_.v, E};
        for (int j = 0; j < 4; j++) std::fill(q.begin() + (size_t)j * nc_, q.begin() + (size_t)(j + 1) * nc_, qq[j]);
        int rc = upload_state(q.data());
        if (rc) return rc;
        init_prims_ = true;
        return FV2D_OK;
    }

    int upload_state(const double* q) {
        FV2D_CUDA(staged_h2d(dstage_, q, 8 * 4 * (size_t)nc_, host_stage_, stream_, stage_free_));
        launch(K_STATE_IN, nc_, [&](int gr) { k_state_in<T><<<gr, 256, 0, stream_>>>(nc_, n2o_, dstage_, Q_[0], Qlo_); });
        // fresh face histories: -101 sentinel for the limiter, initial Vn_avg/c_avg for dt
        FV2D_CUDA(cudaMemsetAsync(smax_, 0, 64, stream_));
        launch(K_SPECTRAL, nc_, [&](int gr) {
            k_spectral_init<T><<<gr, 256, 0, stream_>>>(nc_, inc_off_, inc_, g_.area, S_, smax_, k_);
        });
        FV2D_CUDA(cudaGetLastError());
        FV2D_CUDA(cudaStreamSynchronize(stream_));
        stage_ = 0;
        fresh_ = true;
        init_prims_ = false;
        return FV2D_OK;
    }

    int set_state(const double* q) override { return upload_state(q); }

    // Qbar only; face histories and the stage counter are kept (the run continues).
    int load_state(const double* q) override {
        if (stage_ != 0) { err_ = "load_state between iterations only (stage counter is not 0)"; return FV2D_ERR_ARG; }
        FV2D_CUDA(staged_h2d(dstage_, q, 8 * 4 * (size_t)nc_, host_stage_, stream_, stage_free_));
        launch(K_STATE_IN, nc_, [&](int gr) { k_state_in<T><<<gr, 256, 0, stream_>>>(nc_, n2o_, dstage_, Q_[0], Qlo_); });
        FV2D_CUDA(cudaGetLastError());
        init_prims_ = false;
        return FV2D_OK;
    }

    int stage() override {
        const int s = stage_;
        Q4<T>* qin = Q_[s];
        const int p = (s + 2) % 3;
        if (order2_) {
            constexpr int B = kStageBlock<T>;
            launch(K_GRADIENT, nc_, [&](int gr) {
                if (squeeze_)
                    k_gradient<T, true><<<gr, B, 0, stream_>>>(nc_, dm_, qin, Q_[p], G_[p], G_[s], k_, fresh_ ? 1 : 0,
                                                              init_prims_ ? 1 : 0);
                else
                    k_gradient<T, false><<<gr, B, 0, stream_>>>(nc_, dm_, qin, Q_[p], G_[p], G_[s], k_, fresh_ ? 1 : 0,
                                                               init_prims_ ? 1 : 0);
            }, B);
        }
        launch(K_FACE, nf_, [&](int gr) { launch_face(gr, qin, G_[s], s == 2); }, kStageBlock<T>);
        if (s == 2) FV2D_CUDA(cudaMemsetAsync(smax_, 0, sizeof(T), stream_));
        Q4<T>* rout = (store_every_ || s == 2) ? R_ : nullptr;
        launch(K_UPDATE, nc_, [&](int gr) {
            if (s == 0)
                k_update<T, 0><<<gr, FV2D_UPD_BLOCK, 0, stream_>>>(nc_, dm_, t_, s_, Q_[0], Q_[1], Q_[2], dt_, S_, smax_, rout, flag_, k_, global_dt_, D_, Qlo_);
            else if (s == 1)
                k_update<T, 1><<<gr, FV2D_UPD_BLOCK, 0, stream_>>>(nc_, dm_, t_, s_, Q_[0], Q_[1], Q_[2], dt_, S_, smax_, rout, flag_, k_, global_dt_, D_, Qlo_);
            else
                k_update<T, 2><<<gr, FV2D_UPD_BLOCK, 0, stream_>>>(nc_, dm_, t_, s_, Q_[0], Q_[1], Q_[2], dt_, S_, smax_, rout, flag_, k_, global_dt_, D_, Qlo_);
        }, FV2D_UPD_BLOCK);
        FV2D_CUDA(cudaGetLastError());
        if (s == 0) { fresh_ = false; init_prims_ = false; }
        last_stage_ = s;
        stage_ = (s + 1) % 3;
        return FV2D_OK;
    }

    int step(int iterations) override {
        if (iterations < 0) { err_ = "negative iteration count"; return FV2D_ERR_ARG; }
        int rc;
        int done = 0;
        if (stage_ != 0) {   // finish a partially advanced iteration
            while (stage_ != 0) if ((rc = stage())) return rc;
            done = 1;
        }
        for (int it = done; it < iterations; it++) {
            const bool eager = !graphs_ || timing_ || fresh_ || init_prims_;
            if (eager) {
                for (int s = 0; s < 3; s++) if ((rc = stage())) return rc;
                continue;
            }
            if (!graph_exec_ || graph_store_every_ != store_every_) {
                if ((rc = capture_graph())) return rc;
            }
            FV2D_CUDA(cudaGraphLaunch(graph_exec_, stream_));
            last_stage_ = 2;
        }
        return FV2D_OK;
    }

    int capture_graph() {
        if (graph_exec_) { cudaGraphExecDestroy(graph_exec_); graph_exec_ = nullptr; }
        cudaGraph_t graph;
        FV2D_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        int rc = FV2D_OK;
        for (int s = 0; s < 3 && !rc; s++) rc = stage();
        cudaError_t e = cudaStreamEndCapture(stream_, &graph);
        if (rc) return rc;
        if (e != cudaSuccess) { err_ = std::string("graph capture: ") + cudaGetErrorString(e); return FV2D_ERR_CUDA; }
        e = cudaGraphInstantiate(&graph_exec_, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) { graph_exec_ = nullptr; err_ = std::string("graph instantiate: ") + cudaGetErrorString(e); return FV2D_ERR_CUDA; }
        graph_store_every_ = store_every_;
        return FV2D_OK;
    }

    int get_field(int field, double* out) override {
        int rc = synchronize();
        if (rc && rc != FV2D_ERR_STATE) return rc;
        const void* src = nullptr;
        int ncomp = 4;
        switch (field) {
            case FV2D_F_QBAR: src = Q_[0]; break;
            case FV2D_F_QSTAR: src = (last_stage_ == 0) ? Q_[1] : Q_[2]; break;
            case FV2D_F_RES: src = R_; break;
            case FV2D_F_DT: src = dt_; ncomp = 1; break;
            case FV2D_F_QBAR_GRAD: src = G_[0]; ncomp = 8; break;
            case FV2D_F_QSTAR_GRAD:
                ncomp = 8;
                if (last_stage_ == 0 || last_stage_ < 0 || !order2_) {
                    std::fill(out, out + 8 * (size_t)nc_, 0.0);
                    return FV2D_OK;
                }
                src = G_[last_stage_];
                break;
            default: {
                const int n = mesh_field(mesh_, field, out);
                if (n < 0) { err_ = "unknown field id"; return FV2D_ERR_ARG; }
                return FV2D_OK;
            }
        }
        if ((field == FV2D_F_QBAR_GRAD) && !order2_) { std::fill(out, out + 8 * (size_t)nc_, 0.0); return FV2D_OK; }
        if (ncomp == 1)
            launch(K_STATE_OUT, nc_, [&](int gr) { k_scalar_out<T><<<gr, 256, 0, stream_>>>(nc_, n2o_, (const T*)src, dstage_); });
        else
            launch(K_STATE_OUT, nc_, [&](int gr) {
                k_state_out<T><<<gr, 256, 0, stream_>>>(nc_, ncomp, n2o_, (const Q4<T>*)src, dstage_,
                                                         field == FV2D_F_QBAR ? Qlo_ : nullptr);
            });
        const size_t bytes = 8 * (size_t)ncomp * nc_;
        FV2D_CUDA(staged_d2h(out, dstage_, bytes, host_stage_, stream_, copy_events_));
        return rc;
    }

    int residual_norm(double out[4]) override {
        launch(K_NORM, nc_, [&](int) { k_res_norm_partial<T><<<nred_, 256, 0, stream_>>>(nc_, R_, part_); });
        FV2D_CUDA(cudaMemcpyAsync(host_stage_, part_, 8 * 4 * (size_t)nred_, cudaMemcpyDeviceToHost, stream_));
        int rc = synchronize();
        const double* p = (const double*)host_stage_;
        double acc[4] = {0, 0, 0, 0};
        for (int b = 0; b < nred_; b++) for (int j = 0; j < 4; j++) acc[j] += p[4 * b + j];
        for (int j = 0; j < 4; j++) out[j] = std::sqrt(acc[j]);
        return rc;
    }

    int synchronize() override {
        FV2D_CUDA(cudaStreamSynchronize(stream_));
        int flag = 0;
        FV2D_CUDA(cudaMemcpy(&flag, flag_, sizeof(int), cudaMemcpyDeviceToHost));
        if (flag) { err_ = "non-physical state (rho <= 0, E <= 0 or NaN) produced by an update"; return FV2D_ERR_STATE; }
        return FV2D_OK;
    }

    int set_store_residual(int every) override { store_every_ = every != 0; return FV2D_OK; }
    int set_graphs(int enable) override { graphs_ = enable != 0; return FV2D_OK; }
    int set_timing(int enable) override {
        timing_ = enable != 0;
        for (int i = 0; i < K_COUNT; i++) { ms_[i] = 0; launches_[i] = 0; }
        return FV2D_OK;
    }
    int kernel_times(double* ms, int* launches) override {
        FV2D_CUDA(cudaStreamSynchronize(stream_));
        for (auto& p : pending_) {
            float t = 0;
            cudaEventElapsedTime(&t, p.a, p.b);
            ms_[p.kid] += t;
            launches_[p.kid] += 1;
            free_events_.push_back(p.a);
            free_events_.push_back(p.b);
        }
        pending_.clear();
        for (int i = 0; i < K_COUNT; i++) { ms[i] = ms_[i]; launches[i] = launches_[i]; }
        return FV2D_OK;
    }
    void* stream() override { return (void*)stream_; }
    long long device_bytes() const override { return (long long)arena_bytes_; }

private:
    void launch_face(int gr, const Q4<T>* qin, const Q4<T>* G, bool last) {
#define FV2D_FACE(O2, NS, LAST) \
    k_face<T, O2, NS, LAST><<<gr, kStageBlock<T>, 0, stream_>>>(nf_, dm_, qin, G, t_, s_, k_, init_prims_ ? 1 : 0)
        if (order2_) {
            if (ns_) { if (last) FV2D_FACE(true, true, true); else FV2D_FACE(true, true, false); }
            else { if (last) FV2D_FACE(true, false, true); else FV2D_FACE(true, false, false); }
        } else {
            if (last) FV2D_FACE(false, false, true); else FV2D_FACE(false, false, false);
        }
#undef FV2D_FACE
    }

    template <class F>
    void launch(int kid, int n, F&& fn, int block = 256) {
        const int gr = (n + block - 1) / block;
        if (!timing_) { fn(gr > 0 ? gr : 1); return; }
        Pending p;
        p.kid = kid;
        p.a = get_event();
        p.b = get_event();
        cudaEventRecord(p.a, stream_);
        fn(gr > 0 ? gr : 1);
        cudaEventRecord(p.b, stream_);
        pending_.push_back(p);
    }
    cudaEvent_t get_event() {
        if (!free_events_.empty()) { cudaEvent_t e = free_events_.back(); free_events_.pop_back(); return e; }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }

    struct Pending { int kid; cudaEvent_t a, b; };

    fv2d_case cs_{};
    Consts<T> k_{};
    FaceGeo<T> g_{};
    DevMesh<T> dm_{};
    int nc_ = 0, nf_ = 0, ninc_ = 0, nred_ = 0;
    bool order2_ = false, ns_ = false, squeeze_ = false;
    int global_dt_ = 0;
    bool fresh_ = true, init_prims_ = true, store_every_ = false, graphs_ = true, timing_ = false;
    bool graph_store_every_ = false;
    int last_stage_ = -1;
    cudaStream_t stream_ = nullptr;
    cudaGraphExec_t graph_exec_ = nullptr;
    void* arena_ = nullptr;
    size_t arena_bytes_ = 0;
    void* host_stage_ = nullptr;
    std::vector<cudaEvent_t> copy_events_;   // one per staged D2H chunk
    cudaEvent_t stage_free_ = nullptr;       // the staging buffer's last H2D has been read
    size_t staging_bytes_ = 0;
    Q4<T>* Q_[3] = {nullptr, nullptr, nullptr};
    Q4<T>* G_[3] = {nullptr, nullptr, nullptr};
    Q4<T>* R_ = nullptr;
    Q4<T>* D_ = nullptr;     // FP32 only: RK increment in delta form
    Q4<T>* Qlo_ = nullptr;   // FP32 only: compensation term of Qn
    Q4<T>* t_ = nullptr;
    T *dt_ = nullptr, *S_ = nullptr, *vol_ = nullptr, *s_ = nullptr, *smax_ = nullptr;
    double *Ixx_ = nullptr, *Iyy_ = nullptr, *Ixy_ = nullptr, *dstage_ = nullptr, *part_ = nullptr;
    int *inc_off_ = nullptr, *inc_ = nullptr, *nbr_ = nullptr, *fc1_ = nullptr, *fc2_ = nullptr, *qcell_ = nullptr;
    int *n2o_ = nullptr, *flag_ = nullptr;
    std::vector<Pending> pending_;
    std::vector<cudaEvent_t> free_events_;
    double ms_[K_COUNT] = {0};
    int launches_[K_COUNT] = {0};
};

#undef FV2D_CUDA

}  // namespace fv2d
