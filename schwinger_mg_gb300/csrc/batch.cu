// Many independent lattices of uneven size solved together on one GPU.
//
// Each lattice owns a context (its own CUDA stream, reduction scratch and
// staging), its gauge field, Dirac operator, MG hierarchy and fields.  A pool
// of host worker threads takes lattices from one work queue, largest first
// (longest-processing-time order), and drives each lattice's setup or solve on
// that lattice's stream, so up to n_workers lattices run concurrently and the
// small lattices fill the SMs the large ones leave idle.  Inside a lattice the
// work is the library's own batched path: the right-hand sides of a lattice
// are solved together by GCR with the MG preconditioner (mixed FP32/FP64 for
// an F32 hierarchy), then the pseudofermion force of every right-hand side is
// accumulated, F = sum_j F(X_j) for S = sum_j phi_j^dag (D^dag D)^-1 phi_j
// (fermion_force, reference src/hmc_forces.cpp:134-194).
#include "smg_internal.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <numeric>
#include <thread>
#include <vector>

smg_status smg_fermion_force_dev(smg_dirac* d, const smg_field* X, double* F_dev);
void smg_mg_set_persistent_internal(smg_mg* mg, bool on);

struct smg_batch {
    int device = 0;
    int n_workers = 1;
    struct Lat {
        int L = 0, nrhs = 0;
        double mass = 0, r = 1, c_sw = 0, mu = 0;
        smg_context* ctx = nullptr;
        smg_gauge* g = nullptr;
        smg_dirac* d = nullptr;
        smg_mg* mg = nullptr;
        smg_field* b = nullptr;
        smg_field* x = nullptr;
        smg_field* x1 = nullptr;  // one right-hand side of x for the force
        double* F = nullptr;      // device force accumulator [mu][s]
        double* Fj = nullptr;
        const double* h_rhs = nullptr;
        double* h_x = nullptr;
        double* h_force = nullptr;
        smg_status status = SMG_OK;
        smg_solve_result res{};
        double seconds = 0;
    };
    std::vector<Lat> lat;
};

namespace {

__global__ void k_accumulate(double* __restrict__ F, const double* __restrict__ f, int n, int first) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) F[i] = first ? f[i] : F[i] + f[i];
}

// runs fn(lattice index) for every lattice on the worker pool, largest lattice first
template <typename Fn>
void run_pool(smg_batch* b, Fn fn) {
    std::vector<int> order(b->lat.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int i, int j) {
        return (int64_t)b->lat[i].L * b->lat[i].L * b->lat[i].nrhs > (int64_t)b->lat[j].L * b->lat[j].L * b->lat[j].nrhs;
    });
    std::atomic<size_t> next{0};
    auto worker = [&]() {
        cudaSetDevice(b->device);
        for (;;) {
            const size_t k = next.fetch_add(1);
            if (k >= order.size()) break;
            fn(order[k]);
        }
    };
    const int nw = std::max(1, std::min<int>(b->n_workers, (int)order.size()));
    std::vector<std::thread> th;
    for (int w = 1; w < nw; ++w) th.emplace_back(worker);
    worker();
    for (auto& t : th) t.join();
}

smg_status solve_one(smg_batch::Lat& t, int max_iter, double tol, int trunc, int with_force, int host_io) {
    smg_context* ctx = t.ctx;
    if (host_io && t.h_rhs) SMG_TRY(smg_field_upload_async(t.b, t.h_rhs));
    smg_solve_result r{};
    smg_status st = smg_gcr_solve(t.d, t.mg, t.b, t.x, max_iter, tol, trunc, 0, &r);
    t.res = r;
    if (st != SMG_OK) return st;
    if (with_force) {
        const Geom g = t.x->g;
        const int n = 2 * g.V;
        for (int j = 0; j < t.nrhs; ++j) {
            // column j of x: one 32-byte spinor per site at pitch nrhs * 32 bytes
            SMG_CUDA(ctx, cudaMemcpy2DAsync(t.x1->data, 2 * sizeof(cx<double>),
                                            (const char*)t.x->data + (size_t)j * 2 * sizeof(cx<double>),
                                            (size_t)t.nrhs * 2 * sizeof(cx<double>), 2 * sizeof(cx<double>), g.V,
                                            cudaMemcpyDeviceToDevice, ctx->stream));
            SMG_TRY(smg_fermion_force_dev(t.d, t.x1, t.Fj));
            k_accumulate<<<(n + 255) / 256, 256, 0, ctx->stream>>>(t.F, t.Fj, n, j == 0 ? 1 : 0);
            count_launch(ctx);
            SMG_CHECK_LAUNCH(ctx);
        }
    }
    if (host_io) {
        if (t.h_x) SMG_TRY(smg_field_download_async(t.x, t.h_x));
        if (with_force && t.h_force)
            SMG_CUDA(ctx, cudaMemcpyAsync(t.h_force, t.F, (size_t)2 * t.x->g.V * sizeof(double),
                                          cudaMemcpyDeviceToHost, ctx->stream));
    }
    SMG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SMG_OK;
}

void free_lat(smg_batch::Lat& t) {
    if (t.ctx) cudaStreamSynchronize(t.ctx->stream);
    smg_mg_destroy(t.mg);
    smg_field_destroy(t.b);
    smg_field_destroy(t.x);
    smg_field_destroy(t.x1);
    if (t.F) cudaFree(t.F);
    if (t.Fj) cudaFree(t.Fj);
    smg_dirac_destroy(t.d);
    smg_gauge_destroy(t.g);
    smg_context_destroy(t.ctx);
    t = smg_batch::Lat{};
}

}  // namespace

extern "C" {

SMG_API smg_status smg_batch_create(int device, int n_workers, smg_batch** out) {
    if (!out || n_workers < 1 || n_workers > 256) return SMG_BAD_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return SMG_DEVICE_ERROR;
    smg_batch* b = new smg_batch();
    b->device = device;
    b->n_workers = n_workers;
    *out = b;
    return SMG_OK;
}

SMG_API smg_status smg_batch_destroy(smg_batch* b) {
    if (!b) return SMG_OK;
    for (auto& t : b->lat) free_lat(t);
    delete b;
    return SMG_OK;
}

SMG_API smg_status smg_batch_add(smg_batch* b, int L, const double* U, double mass, double wilson_r, double c_sw,
                                 double mu_t, int nrhs, int* id) {
    if (!b || !U || L < 4 || L % 2 || nrhs < 1) return SMG_BAD_ARG;
    smg_batch::Lat t;
    t.L = L;
    t.nrhs = nrhs;
    t.mass = mass;
    t.r = wilson_r;
    t.c_sw = c_sw;
    t.mu = mu_t;
    smg_status st = smg_context_create(b->device, nullptr, &t.ctx);
    if (st == SMG_OK) st = smg_gauge_create(t.ctx, L, U, &t.g);
    if (st == SMG_OK) st = smg_dirac_create(t.g, mass, wilson_r, c_sw, mu_t, &t.d);
    if (st == SMG_OK) st = smg_field_create(t.ctx, L, nrhs, SMG_F64, &t.b);
    if (st == SMG_OK) st = smg_field_create(t.ctx, L, nrhs, SMG_F64, &t.x);
    if (st == SMG_OK) st = smg_field_create(t.ctx, L, 1, SMG_F64, &t.x1);
    if (st == SMG_OK && (cudaMalloc(&t.F, (size_t)2 * L * L * sizeof(double)) != cudaSuccess ||
                         cudaMalloc(&t.Fj, (size_t)2 * L * L * sizeof(double)) != cudaSuccess))
        st = SMG_NO_MEMORY;
    if (st != SMG_OK) {
        free_lat(t);
        return st;
    }
    b->lat.push_back(t);
    if (id) *id = (int)b->lat.size() - 1;
    return SMG_OK;
}

SMG_API smg_status smg_batch_setup(smg_batch* b, const smg_mg_params* p) {
    if (!b || !p) return SMG_BAD_ARG;
    run_pool(b, [&](int i) {
        smg_batch::Lat& t = b->lat[i];
        if (t.mg) {
            smg_mg_destroy(t.mg);
            t.mg = nullptr;
        }
        t.status = smg_mg_create(t.d, p, nullptr, &t.mg);
        if (t.status == SMG_OK) smg_mg_set_persistent_internal(t.mg, false);
        cudaStreamSynchronize(t.ctx->stream);
    });
    for (auto& t : b->lat)
        if (t.status != SMG_OK) return t.status;
    return SMG_OK;
}

SMG_API smg_status smg_batch_bind_host(smg_batch* b, int id, const double* rhs, double* x, double* force) {
    if (!b || id < 0 || id >= (int)b->lat.size()) return SMG_BAD_ARG;
    smg_batch::Lat& t = b->lat[id];
    t.h_rhs = rhs;
    t.h_x = x;
    t.h_force = force;
    if (rhs) SMG_TRY(smg_field_upload(t.b, rhs));
    return SMG_OK;
}

SMG_API smg_status smg_batch_solve(smg_batch* b, int max_iter, double tol, int trunc, int with_force, int host_io,
                                   double* seconds) {
    if (!b || max_iter < 0 || !(tol > 0) || trunc < 1) return SMG_BAD_ARG;
    for (auto& t : b->lat)
        if (!t.mg) return smg_fail(t.ctx, SMG_BAD_ARG, "batch_solve before batch_setup");
    const auto t0 = std::chrono::steady_clock::now();
    run_pool(b, [&](int i) {
        smg_batch::Lat& t = b->lat[i];
        const auto s0 = std::chrono::steady_clock::now();
        t.status = solve_one(t, max_iter, tol, trunc, with_force, host_io);
        t.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - s0).count();
    });
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    smg_status worst = SMG_OK;
    for (auto& t : b->lat)
        if (t.status != SMG_OK && (worst == SMG_OK || worst == SMG_NOT_CONVERGED)) worst = t.status;
    return worst;
}

SMG_API smg_status smg_batch_result(smg_batch* b, int id, smg_solve_result* res, smg_status* status,
                                    double* seconds) {
    if (!b || id < 0 || id >= (int)b->lat.size()) return SMG_BAD_ARG;
    const smg_batch::Lat& t = b->lat[id];
    if (res) *res = t.res;
    if (status) *status = t.status;
    if (seconds) *seconds = t.seconds;
    return SMG_OK;
}

SMG_API smg_status smg_batch_download(smg_batch* b, int id, double* x, double* force) {
    if (!b || id < 0 || id >= (int)b->lat.size()) return SMG_BAD_ARG;
    smg_batch::Lat& t = b->lat[id];
    if (x) SMG_TRY(smg_field_download(t.x, x));
    if (force) {
        SMG_CUDA(t.ctx, cudaMemcpyAsync(force, t.F, (size_t)2 * t.L * t.L * sizeof(double), cudaMemcpyDeviceToHost,
                                        t.ctx->stream));
        SMG_CUDA(t.ctx, cudaStreamSynchronize(t.ctx->stream));
    }
    return SMG_OK;
}

SMG_API smg_status smg_batch_kernel_launches(smg_batch* b, uint64_t* n) {
    if (!b || !n) return SMG_BAD_ARG;
    uint64_t t = 0;
    for (const auto& l : b->lat) t += l.ctx ? l.ctx->launches : 0;
    *n = t;
    return SMG_OK;
}

}  // extern "C"
