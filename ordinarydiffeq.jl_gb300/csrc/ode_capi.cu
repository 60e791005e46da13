// Host runtime of libode_b200.so: the C ABI declared in include/ode_gb300.h.
//
// Responsibilities: validate requests, choose the compiled kernel variant
// (lanes per trajectory, block size), group trajectories of different sizes,
// own the device scratch (work-queue counters, size-class buckets, staging
// buffers), time launches with CUDA events, and run the continuous-batching
// serving loop.  There is no CPU fallback: if a request has no compiled GPU
// variant the call fails with ODE_E_UNSUPPORTED.
#include "ode_gb300.h"
#include "ode_kernels.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

using namespace odegb;

namespace {

thread_local std::string g_tls_error;

const std::vector<KernelVariant>& all_variants() {
    static std::vector<KernelVariant> v = [] {
        std::vector<KernelVariant> out;
        int n = 0;
        const KernelVariant* t = tsit5_variants(&n);
        out.insert(out.end(), t, t + n);
        t = vern7_variants(&n);
        out.insert(out.end(), t, t + n);
        t = rodas_variants(&n);
        out.insert(out.end(), t, t + n);
        return out;
    }();
    return v;
}

int model_nparams(int model) { return model == ODE_MODEL_LINEAR ? 1 : 3; }

// Default lanes per trajectory: one lane for tiny systems (registers hold the
// whole state and stage set), else 4 states per lane so the Vern7 stage set
// stays in registers without spilling.
int default_lanes(int alg, int n) {
    if (n <= 4 || (n <= 8 && alg == ODE_RODAS5P)) return 1;
    return std::min(32, n / 4);
}

const KernelVariant* find_variant(int alg, int model, int prec, int n, int lanes) {
    const KernelVariant* best = nullptr;
    for (const auto& v : all_variants()) {
        if (v.alg != alg || v.model != model || v.prec != prec || v.n != n) continue;
        if (lanes > 0 && v.lanes != lanes) continue;
        if (!best) best = &v;
        if (lanes <= 0 && v.lanes == default_lanes(alg, n)) best = &v;
    }
    return best;
}

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
};

// Stream-scoped device scratch: one for the synchronous API and one per
// serving slot, so concurrent requests never share a work counter or bucket.
struct Ctx {
    cudaStream_t stream = nullptr;
    unsigned long long* d_queue = nullptr;  // [0,8) per-class work counters, [8,16) counts, [16,24) cursors
    long long* d_order = nullptr;           // bucketed trajectory indices
    size_t order_cap = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaStream_t class_streams[5] = {};
    cudaEvent_t class_events[5] = {};
};

struct Request;

}  // namespace

struct ode_handle {
    int device = 0;
    int sm_count = 0;
    size_t budget = 0;
    std::string err;
    int* h_abort = nullptr;                 // pinned, mapped: host writes, kernels poll
    int* d_abort = nullptr;
    double last_ms = 0.0;
    std::atomic<long long> launches{0};
    Ctx main;
    // staging for the synchronous host API
    DevBuf b_u0, b_p, b_tspan, b_saveat, b_t, b_u, b_ns, b_rc, b_st, b_npt;
    std::mutex api_mu;
    // serving
    std::mutex mu;
    std::condition_variable cv;
    std::deque<std::shared_ptr<Request>> pending;
    std::vector<std::shared_ptr<Request>> running;
    std::map<uint64_t, std::shared_ptr<Request>> tickets;
    std::thread worker;
    bool stop = false;
    bool worker_started = false;
    int slots = 8;
    uint64_t next_ticket = 1;
    size_t hbm_in_use = 0;
    long long n_submitted = 0, n_admitted = 0, n_completed = 0, n_rejected = 0;
    std::vector<Ctx> slot_ctx;
    std::vector<int> slot_busy;
};

namespace {

int fail(ode_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    g_tls_error = msg;
    return code;
}

#define CUDA_TRY(h, call)                                                                   \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(h, ODE_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int grow(ode_handle* h, DevBuf& b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.cap >= bytes) return ODE_OK;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) return fail(h, ODE_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    b.cap = bytes;
    return ODE_OK;
}

int validate(ode_handle* h, const ode_problem_desc* d, const ode_options* o, int64_t N) {
    if (!h || !d || !o) return fail(h, ODE_E_INVALID, "null handle, problem or options");
    if (N < 0) return fail(h, ODE_E_INVALID, "negative trajectory count");
    if (d->alg_id < ODE_TSIT5 || d->alg_id > ODE_RODAS5P) return fail(h, ODE_E_INVALID, "unknown alg_id");
    if (d->model_id < ODE_MODEL_LINEAR || d->model_id > ODE_MODEL_BRUSSELATOR_1D)
        return fail(h, ODE_E_INVALID, "unknown model_id");
    if (d->precision != ODE_PREC_FP64 && d->precision != ODE_PREC_MIXED)
        return fail(h, ODE_E_INVALID, "unknown precision");
    if (d->n_states <= 0) return fail(h, ODE_E_INVALID, "n_states must be positive");
    if (d->n_params != model_nparams(d->model_id))
        return fail(h, ODE_E_INVALID, "n_params does not match the model");
    if ((d->model_id == ODE_MODEL_LORENZ || d->model_id == ODE_MODEL_ROBERTSON) && d->n_states != 3)
        return fail(h, ODE_E_INVALID, "this model has 3 states");
    if (!(o->reltol > 0) || !(o->abstol >= 0)) return fail(h, ODE_E_INVALID, "tolerances must be positive");
    if (o->nsave < 0) return fail(h, ODE_E_INVALID, "negative nsave");
    return ODE_OK;
}

EnsembleArgs make_args(ode_handle* h, const ode_problem_desc* d, const ode_options* o, int64_t N,
                       const double* u0, const double* p, const double* tspan, const double* saveat,
                       double* t_out, double* u_out, int32_t* nsaved, int32_t* retcode, OdeStatsDev* stats) {
    EnsembleArgs a;
    std::memset(&a, 0, sizeof(a));
    a.N = N;
    a.count = N;
    a.order = nullptr;
    a.nmax = d->n_states;
    a.u0 = u0;
    a.p = p;
    a.tspan = tspan;
    a.saveat = saveat;
    a.nsave = o->nsave;
    a.saveat_per_traj = o->saveat_per_traj;
    a.nsave_cap = o->nsave + 2;
    a.t_out = t_out;
    a.u_out = u_out;
    a.nsaved = nsaved;
    a.retcode = retcode;
    a.stats = stats;
    a.reltol = o->reltol;
    a.abstol = o->abstol;
    a.dtmax = o->dtmax;
    a.dtmin = o->dtmin;
    a.dt = o->dt;
    a.maxiters = o->maxiters > 0 ? o->maxiters : 1000000;
    a.save_start = o->save_start;
    a.save_end = o->save_end;
    a.save_end_user = o->save_end_user;
    a.saveat_given = o->nsave > 0;
    a.saveat_scalar = o->saveat_scalar;
    a.qmax_first_step = o->qmax_first_step;
    a.qmax = o->qmax;
    // Register-resident Rosenbrock solves (n <= 8) default to no refinement:
    // their FP32 LU error is far below the tolerance; sweeps are available on request.
    a.ir_sweeps = o->ir_sweeps < 0 ? 0 : o->ir_sweeps;
    a.abort_flag = h->d_abort;
    return a;
}

// Bucket trajectories by state count on the device (histogram + scatter).
__global__ void bucket_count(const int32_t* npt, long long N, unsigned long long* counts) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    int n = npt[j];
    int c = n <= 4 ? 0 : n <= 8 ? 1 : n <= 16 ? 2 : n <= 32 ? 3 : 4;
    atomicAdd(&counts[c], 1ull);
}
__global__ void bucket_scatter(const int32_t* npt, long long N, unsigned long long* cursor, long long* order) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    int n = npt[j];
    int c = n <= 4 ? 0 : n <= 8 ? 1 : n <= 16 ? 2 : n <= 32 ? 3 : 4;
    unsigned long long slot = atomicAdd(&cursor[c], 1ull);
    order[slot] = j;
}

constexpr int kClassN[5] = {4, 8, 16, 32, 64};
constexpr int kBlock = 128;

int launch_variant(ode_handle* h, const KernelVariant* v, EnsembleArgs a, int scheduler, int block,
                   unsigned long long* queue, cudaStream_t s) {
    if (v->lanes > 1 && block % 32 != 0) block = kBlock;
    if (a.count <= 0) return ODE_OK;
    if (block <= 0) block = kBlock;
    if (block > 128) block = 128;
    long long groups = a.count;
    bool persistent = scheduler == 2;
    int grid;
    if (persistent) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, v->fn, block, 0);
        if (per_sm <= 0) per_sm = 1;
        long long want = (groups * v->lanes + block - 1) / block;
        grid = (int)std::min<long long>((long long)per_sm * h->sm_count, want);
        if (grid < 1) grid = 1;
        CUDA_TRY(h, cudaMemsetAsync(queue, 0, sizeof(unsigned long long), s));
        a.queue = queue;
        a.persistent = 1;
    } else {
        long long threads = groups * v->lanes;
        grid = (int)((threads + block - 1) / block);
        a.persistent = 0;
    }
    v->launch(a, grid, block, 0, s);
    h->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(h, ODE_E_CUDA, std::string("launch ") + v->name + ": " + cudaGetErrorString(e));
    return ODE_OK;
}

int ctx_init(ode_handle* h, Ctx& c, cudaStream_t s) {
    if (s) c.stream = s;
    else CUDA_TRY(h, cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    CUDA_TRY(h, cudaMalloc(&c.d_queue, 32 * sizeof(unsigned long long)));
    CUDA_TRY(h, cudaMemset(c.d_queue, 0, 32 * sizeof(unsigned long long)));
    CUDA_TRY(h, cudaEventCreate(&c.ev0));
    CUDA_TRY(h, cudaEventCreate(&c.ev1));
    for (int k = 0; k < 5; ++k) {
        CUDA_TRY(h, cudaStreamCreateWithFlags(&c.class_streams[k], cudaStreamNonBlocking));
        CUDA_TRY(h, cudaEventCreateWithFlags(&c.class_events[k], cudaEventDisableTiming));
    }
    return ODE_OK;
}

void ctx_free(Ctx& c) {
    if (c.d_queue) cudaFree(c.d_queue);
    if (c.d_order) cudaFree(c.d_order);
    for (int k = 0; k < 5; ++k) {
        if (c.class_streams[k]) cudaStreamDestroy(c.class_streams[k]);
        if (c.class_events[k]) cudaEventDestroy(c.class_events[k]);
    }
    if (c.ev0) cudaEventDestroy(c.ev0);
    if (c.ev1) cudaEventDestroy(c.ev1);
    if (c.stream) cudaStreamDestroy(c.stream);
    c = Ctx();
}

// Enqueue the whole ensemble on stream s using the scratch of ctx c.  All
// pointers are device pointers.
int run_ensemble(ode_handle* h, Ctx& c, const ode_problem_desc* d, const ode_options* o, int64_t N,
                 const int32_t* npt_dev, const double* u0, const double* p, const double* tspan,
                 const double* saveat, double* t_out, double* u_out, int32_t* nsaved, int32_t* retcode,
                 OdeStatsDev* stats, cudaStream_t s) {
    EnsembleArgs a = make_args(h, d, o, N, u0, p, tspan, saveat, t_out, u_out, nsaved, retcode, stats);
    int scheduler = o->scheduler;
    if (N == 0) return ODE_OK;
    if (npt_dev == nullptr) {
        const KernelVariant* v = find_variant(d->alg_id, d->model_id, d->precision, d->n_states, o->lanes_per_traj);
        if (!v) {
            char buf[160];
            std::snprintf(buf, sizeof buf, "no compiled kernel for alg %d model %d precision %d n %d lanes %d",
                          d->alg_id, d->model_id, d->precision, d->n_states, o->lanes_per_traj);
            return fail(h, ODE_E_UNSUPPORTED, buf);
        }
        if (scheduler == 0) scheduler = 1;
        CUDA_TRY(h, cudaEventRecord(c.ev0, s));
        int rc = launch_variant(h, v, a, scheduler, o->block_size, c.d_queue, s);
        if (rc) return rc;
        CUDA_TRY(h, cudaEventRecord(c.ev1, s));
        return ODE_OK;
    }
    // Uneven sizes: bucket by state count, then one persistent kernel per size
    // class, run concurrently on the handle's class streams.
    if (d->model_id != ODE_MODEL_DUFFING_CHAIN)
        return fail(h, ODE_E_UNSUPPORTED, "per-trajectory sizes are supported for DUFFING_CHAIN");
    if ((size_t)N > c.order_cap) {
        if (c.d_order) cudaFree(c.d_order);
        c.d_order = nullptr;
        c.order_cap = 0;
        CUDA_TRY(h, cudaMalloc(&c.d_order, sizeof(long long) * (size_t)N));
        c.order_cap = (size_t)N;
    }
    unsigned long long* counts = c.d_queue + 8;
    unsigned long long* cursor = c.d_queue + 16;
    CUDA_TRY(h, cudaMemsetAsync(counts, 0, 8 * sizeof(unsigned long long), s));
    int gb = (int)((N + 255) / 256);
    bucket_count<<<gb, 256, 0, s>>>(npt_dev, N, counts);
    unsigned long long hc[8] = {0};
    CUDA_TRY(h, cudaMemcpyAsync(hc, counts, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(h, cudaStreamSynchronize(s));
    unsigned long long off[5];
    unsigned long long acc = 0;
    for (int k = 0; k < 5; ++k) { off[k] = acc; acc += hc[k]; }
    CUDA_TRY(h, cudaMemcpyAsync(cursor, off, 5 * sizeof(unsigned long long), cudaMemcpyHostToDevice, s));
    bucket_scatter<<<gb, 256, 0, s>>>(npt_dev, N, cursor, c.d_order);
    h->launches += 2;
    CUDA_TRY(h, cudaEventRecord(c.ev0, s));
    if (scheduler == 0) scheduler = 2;
    for (int k = 0; k < 5; ++k) {
        if (hc[k] == 0) continue;
        const KernelVariant* v = find_variant(d->alg_id, d->model_id, d->precision, kClassN[k], 0);
        if (!v) return fail(h, ODE_E_UNSUPPORTED, "no compiled kernel for a Duffing size class");
        CUDA_TRY(h, cudaStreamWaitEvent(c.class_streams[k], c.ev0, 0));
        EnsembleArgs ac = a;
        ac.order = c.d_order + off[k];
        ac.count = (long long)hc[k];
        int rc = launch_variant(h, v, ac, scheduler, o->block_size, c.d_queue + k, c.class_streams[k]);
        if (rc) return rc;
        CUDA_TRY(h, cudaEventRecord(c.class_events[k], c.class_streams[k]));
        CUDA_TRY(h, cudaStreamWaitEvent(s, c.class_events[k], 0));
    }
    CUDA_TRY(h, cudaEventRecord(c.ev1, s));
    return ODE_OK;
}

size_t save_cap(const ode_options* o) { return (size_t)o->nsave + 2; }

}  // namespace

// ============================================================== serving
namespace {

// One queued or running serving request.  Inputs are copied at submit time so
// the caller may reuse its input buffers; outputs go to the caller's buffers.
struct Request {
    uint64_t ticket = 0;
    ode_problem_desc d;
    ode_options o;
    int64_t N = 0;
    std::vector<double> u0, p, tspan, saveat;
    std::vector<int32_t> npt;
    double* t_out = nullptr;
    double* u_out = nullptr;
    int32_t* nsaved = nullptr;
    int32_t* retcode = nullptr;
    ode_stats* stats = nullptr;
    int state = 0;  // 0 queued, 1 running, 2 done
    int status = ODE_OK;
    int slot = -1;
    size_t bytes = 0;
    void* dmem = nullptr;      // one device block for inputs and outputs
    void* hout = nullptr;      // pinned staging for outputs
    cudaEvent_t done_ev = nullptr;
};

size_t request_bytes(const Request& r) {
    size_t n = (size_t)r.d.n_states, np = (size_t)r.d.n_params, cap = (size_t)r.o.nsave + 2, N = (size_t)r.N;
    size_t in = (n + np + 2) * N * 8 + r.saveat.size() * 8 + r.npt.size() * 4;
    size_t out = cap * N * 8 + cap * n * N * 8 + N * 8 + N * sizeof(ode_stats);
    return in + out + 1024;
}

size_t output_bytes(const Request& r) {
    size_t n = (size_t)r.d.n_states, cap = (size_t)r.o.nsave + 2, N = (size_t)r.N;
    return cap * N * 8 + cap * n * N * 8 + N * 8 + N * sizeof(ode_stats) + 256;
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Admit r on slot k: stage inputs, launch, copy outputs back (all async).
int admit(ode_handle* h, Request& r, int k) {
    Ctx& c = h->slot_ctx[k];
    cudaStream_t s = c.stream;
    const size_t n = (size_t)r.d.n_states, np = (size_t)r.d.n_params, N = (size_t)r.N, cap = (size_t)r.o.nsave + 2;
    CUDA_TRY(h, cudaMallocAsync(&r.dmem, r.bytes, s));
    char* base = (char*)r.dmem;
    size_t off = 0;
    auto take = [&](size_t bytes) { char* q = base + off; off += align256(bytes); return q; };
    double* du0 = (double*)take(n * N * 8);
    double* dp = (double*)take(np * N * 8);
    double* dts = (double*)take(2 * N * 8);
    double* dsv = (double*)take(std::max<size_t>(r.saveat.size(), 1) * 8);
    int32_t* dnpt = r.npt.empty() ? nullptr : (int32_t*)take(N * 4);
    double* dt = (double*)take(cap * N * 8);
    double* du = (double*)take(cap * n * N * 8);
    int32_t* dns = (int32_t*)take(N * 4);
    int32_t* drc = (int32_t*)take(N * 4);
    ode_stats* dst = (ode_stats*)take(N * sizeof(ode_stats));
    CUDA_TRY(h, cudaMemcpyAsync(du0, r.u0.data(), n * N * 8, cudaMemcpyHostToDevice, s));
    CUDA_TRY(h, cudaMemcpyAsync(dp, r.p.data(), np * N * 8, cudaMemcpyHostToDevice, s));
    CUDA_TRY(h, cudaMemcpyAsync(dts, r.tspan.data(), 2 * N * 8, cudaMemcpyHostToDevice, s));
    if (!r.saveat.empty())
        CUDA_TRY(h, cudaMemcpyAsync(dsv, r.saveat.data(), r.saveat.size() * 8, cudaMemcpyHostToDevice, s));
    if (dnpt) CUDA_TRY(h, cudaMemcpyAsync(dnpt, r.npt.data(), N * 4, cudaMemcpyHostToDevice, s));
    int rc = run_ensemble(h, c, &r.d, &r.o, r.N, dnpt, du0, dp, dts, dsv, dt, du, dns, drc, (OdeStatsDev*)dst, s);
    if (rc) return rc;
    CUDA_TRY(h, cudaMallocHost(&r.hout, output_bytes(r)));
    char* ho = (char*)r.hout;
    CUDA_TRY(h, cudaMemcpyAsync(ho, dt, cap * N * 8, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(h, cudaMemcpyAsync(ho + cap * N * 8, du, cap * n * N * 8, cudaMemcpyDeviceToHost, s));
    size_t o2 = cap * N * 8 + cap * n * N * 8;
    CUDA_TRY(h, cudaMemcpyAsync(ho + o2, dns, N * 4, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(h, cudaMemcpyAsync(ho + o2 + N * 4, drc, N * 4, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(h, cudaMemcpyAsync(ho + o2 + N * 8, dst, N * sizeof(ode_stats), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(h, cudaFreeAsync(r.dmem, s));
    r.dmem = nullptr;
    CUDA_TRY(h, cudaEventCreateWithFlags(&r.done_ev, cudaEventDisableTiming));
    CUDA_TRY(h, cudaEventRecord(r.done_ev, s));
    return ODE_OK;
}

void finish(Request& r) {
    const size_t n = (size_t)r.d.n_states, N = (size_t)r.N, cap = (size_t)r.o.nsave + 2;
    if (r.status == ODE_OK && r.hout) {
        char* ho = (char*)r.hout;
        if (r.t_out) std::memcpy(r.t_out, ho, cap * N * 8);
        std::memcpy(r.u_out, ho + cap * N * 8, cap * n * N * 8);
        size_t o2 = cap * N * 8 + cap * n * N * 8;
        std::memcpy(r.nsaved, ho + o2, N * 4);
        std::memcpy(r.retcode, ho + o2 + N * 4, N * 4);
        if (r.stats) std::memcpy(r.stats, ho + o2 + N * 8, N * sizeof(ode_stats));
    }
    if (r.hout) cudaFreeHost(r.hout);
    r.hout = nullptr;
    if (r.done_ev) cudaEventDestroy(r.done_ev);
    r.done_ev = nullptr;
    r.u0.clear(); r.u0.shrink_to_fit();
    r.p.clear(); r.p.shrink_to_fit();
    r.state = 2;
}

// The serving loop: retire finished requests, then admit queued ones (FIFO)
// while a slot is free and the HBM budget allows.  A request larger than the
// whole budget is rejected with ODE_E_NOMEM.
void serve_loop(ode_handle* h) {
    cudaSetDevice(h->device);
    std::unique_lock<std::mutex> lk(h->mu);
    while (!h->stop) {
        bool progressed = false;
        for (size_t i = 0; i < h->running.size();) {
            auto r = h->running[i];
            cudaError_t q = cudaEventQuery(r->done_ev);
            if (q == cudaErrorNotReady) { ++i; continue; }
            if (q != cudaSuccess) r->status = ODE_E_CUDA;
            finish(*r);
            h->slot_busy[r->slot] = 0;
            h->hbm_in_use -= r->bytes;
            h->n_completed++;
            h->running.erase(h->running.begin() + i);
            progressed = true;
        }
        while (!h->pending.empty()) {
            auto r = h->pending.front();
            if (r->bytes > h->budget) {
                h->pending.pop_front();
                r->status = ODE_E_NOMEM;
                r->state = 2;
                h->n_rejected++;
                progressed = true;
                continue;
            }
            int k = -1;
            for (int s = 0; s < (int)h->slot_ctx.size(); ++s)
                if (!h->slot_busy[s]) { k = s; break; }
            if (k < 0 || h->hbm_in_use + r->bytes > h->budget) break;
            h->pending.pop_front();
            r->slot = k;
            h->slot_busy[k] = 1;
            h->hbm_in_use += r->bytes;
            r->state = 1;
            h->n_admitted++;
            int rc = admit(h, *r, k);
            if (rc) {
                r->status = rc;
                cudaStreamSynchronize(h->slot_ctx[k].stream);
                if (r->dmem) cudaFree(r->dmem);
                r->dmem = nullptr;
                finish(*r);
                h->slot_busy[k] = 0;
                h->hbm_in_use -= r->bytes;
                h->n_completed++;
            } else {
                h->running.push_back(r);
            }
            progressed = true;
        }
        if (progressed) h->cv.notify_all();
        if (h->running.empty() && h->pending.empty())
            h->cv.wait(lk, [&] { return h->stop || !h->pending.empty(); });
        else
            h->cv.wait_for(lk, std::chrono::microseconds(50));
    }
}

int ensure_worker(ode_handle* h) {
    if (h->worker_started) return ODE_OK;
    h->slot_ctx.resize(h->slots);
    h->slot_busy.assign(h->slots, 0);
    for (int k = 0; k < h->slots; ++k) {
        int rc = ctx_init(h, h->slot_ctx[k], nullptr);
        if (rc) return rc;
    }
    h->worker = std::thread(serve_loop, h);
    h->worker_started = true;
    return ODE_OK;
}

}  // namespace

// ============================================================== C ABI
extern "C" {

int ode_abi_version(void) { return ODE_ABI_VERSION; }

const char* ode_status_string(int s) {
    switch (s) {
    case ODE_OK: return "ok";
    case ODE_E_INVALID: return "invalid argument";
    case ODE_E_CUDA: return "CUDA error";
    case ODE_E_NOMEM: return "out of device memory";
    case ODE_E_UNSUPPORTED: return "unsupported (no compiled kernel)";
    case ODE_E_BUSY: return "busy";
    case ODE_E_TIMEOUT: return "timeout";
    case ODE_E_NOTFOUND: return "unknown ticket";
    }
    return "unknown status";
}

const char* ode_last_error(const ode_handle* h) { return h ? h->err.c_str() : g_tls_error.c_str(); }

void ode_options_default(ode_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->reltol = 1e-3;
    o->abstol = 1e-6;
    o->maxiters = 1000000;
    o->save_start = 1;
    o->save_end = 1;
    o->save_end_user = -1;
    o->ir_sweeps = -1;
}

int ode_create(int device, size_t hbm_budget, ode_handle** out) {
    if (!out) return fail(nullptr, ODE_E_INVALID, "null output pointer");
    *out = nullptr;
    std::unique_ptr<ode_handle> h(new ode_handle());
    h->device = device;
    CUDA_TRY(h.get(), cudaSetDevice(device));
    CUDA_TRY(h.get(), cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device));
    int rc = ctx_init(h.get(), h->main, nullptr);
    if (rc) return rc;
    CUDA_TRY(h.get(), cudaHostAlloc((void**)&h->h_abort, sizeof(int), cudaHostAllocMapped));
    *h->h_abort = 0;
    CUDA_TRY(h.get(), cudaHostGetDevicePointer((void**)&h->d_abort, h->h_abort, 0));
    size_t freeb = 0, total = 0;
    CUDA_TRY(h.get(), cudaMemGetInfo(&freeb, &total));
    h->budget = hbm_budget ? hbm_budget : (size_t)(0.9 * (double)freeb);
    *out = h.release();
    return ODE_OK;
}

void ode_destroy(ode_handle* h) {
    if (!h) return;
    {
        std::unique_lock<std::mutex> lk(h->mu);
        h->stop = true;
    }
    h->cv.notify_all();
    if (h->worker_started && h->worker.joinable()) h->worker.join();
    cudaSetDevice(h->device);
    cudaDeviceSynchronize();
    for (auto& r : h->running) finish(*r);
    for (DevBuf* b : {&h->b_u0, &h->b_p, &h->b_tspan, &h->b_saveat, &h->b_t, &h->b_u, &h->b_ns, &h->b_rc,
                      &h->b_st, &h->b_npt})
        if (b->p) cudaFree(b->p);
    ctx_free(h->main);
    for (auto& c : h->slot_ctx) ctx_free(c);
    if (h->h_abort) cudaFreeHost(h->h_abort);
    delete h;
}

int ode_solve_ensemble_device(ode_handle* h, const ode_problem_desc* d, const ode_options* o, int64_t N,
                              const int32_t* npt_dev, const double* u0, const double* p, const double* tspan,
                              const double* saveat, double* t_out, double* u_out, int32_t* nsaved,
                              int32_t* retcode, ode_stats* stats, void* cuda_stream) {
    int rc = validate(h, d, o, N);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(h->api_mu);
    CUDA_TRY(h, cudaSetDevice(h->device));
    *h->h_abort = 0;
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : h->main.stream;
    return run_ensemble(h, h->main, d, o, N, npt_dev, u0, p, tspan, saveat, t_out, u_out, nsaved, retcode,
                        (OdeStatsDev*)stats, s);
}

int ode_solve_ensemble(ode_handle* h, const ode_problem_desc* d, const ode_options* o, int64_t N,
                       const int32_t* npt, const double* u0, const double* p, const double* tspan,
                       const double* saveat, double* t_out, double* u_out, int32_t* nsaved, int32_t* retcode,
                       ode_stats* stats) {
    int rc = validate(h, d, o, N);
    if (rc) return rc;
    if (N > 0 && (!u0 || !p || !tspan || !u_out || !nsaved || !retcode))
        return fail(h, ODE_E_INVALID, "null input or output buffer");
    if (o->nsave > 0 && !saveat) return fail(h, ODE_E_INVALID, "nsave > 0 but saveat is null");
    std::lock_guard<std::mutex> lk(h->api_mu);
    CUDA_TRY(h, cudaSetDevice(h->device));
    *h->h_abort = 0;
    const size_t n = (size_t)d->n_states, np = (size_t)d->n_params, cap = save_cap(o);
    const size_t nsv = (size_t)o->nsave * (o->saveat_per_traj ? (size_t)N : 1);
    if ((rc = grow(h, h->b_u0, n * N * 8)) || (rc = grow(h, h->b_p, np * N * 8)) ||
        (rc = grow(h, h->b_tspan, 2 * N * 8)) || (rc = grow(h, h->b_saveat, nsv * 8)) ||
        (rc = grow(h, h->b_t, cap * N * 8)) || (rc = grow(h, h->b_u, cap * n * N * 8)) ||
        (rc = grow(h, h->b_ns, N * 4)) || (rc = grow(h, h->b_rc, N * 4)) ||
        (rc = grow(h, h->b_st, N * sizeof(ode_stats))) || (npt && (rc = grow(h, h->b_npt, N * 4))))
        return rc;
    cudaStream_t s = h->main.stream;
    CUDA_TRY(h, cudaMemcpyAsync(h->b_u0.p, u0, n * N * 8, cudaMemcpyHostToDevice, s));
    CUDA_TRY(h, cudaMemcpyAsync(h->b_p.p, p, np * N * 8, cudaMemcpyHostToDevice, s));
    CUDA_TRY(h, cudaMemcpyAsync(h->b_tspan.p, tspan, 2 * N * 8, cudaMemcpyHostToDevice, s));
    if (nsv) CUDA_TRY(h, cudaMemcpyAsync(h->b_saveat.p, saveat, nsv * 8, cudaMemcpyHostToDevice, s));
    if (npt) CUDA_TRY(h, cudaMemcpyAsync(h->b_npt.p, npt, N * 4, cudaMemcpyHostToDevice, s));
    rc = run_ensemble(h, h->main, d, o, N, npt ? (const int32_t*)h->b_npt.p : nullptr, (const double*)h->b_u0.p,
                      (const double*)h->b_p.p, (const double*)h->b_tspan.p, (const double*)h->b_saveat.p,
                      (double*)h->b_t.p, (double*)h->b_u.p, (int32_t*)h->b_ns.p, (int32_t*)h->b_rc.p,
                      (OdeStatsDev*)h->b_st.p, s);
    if (rc) {
        cudaStreamSynchronize(s);
        return rc;
    }
    if (t_out) CUDA_TRY(h, cudaMemcpyAsync(t_out, h->b_t.p, cap * N * 8, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(h, cudaMemcpyAsync(u_out, h->b_u.p, cap * n * N * 8, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(h, cudaMemcpyAsync(nsaved, h->b_ns.p, N * 4, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(h, cudaMemcpyAsync(retcode, h->b_rc.p, N * 4, cudaMemcpyDeviceToHost, s));
    if (stats) CUDA_TRY(h, cudaMemcpyAsync(stats, h->b_st.p, N * sizeof(ode_stats), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(h, cudaStreamSynchronize(s));
    if (N > 0) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, h->main.ev0, h->main.ev1) == cudaSuccess) h->last_ms = ms;
    }
    return ODE_OK;
}

int ode_submit(ode_handle* h, const ode_problem_desc* d, const ode_options* o, int64_t N, const int32_t* npt,
               const double* u0, const double* p, const double* tspan, const double* saveat, double* t_out,
               double* u_out, int32_t* nsaved, int32_t* retcode, ode_stats* stats, uint64_t* ticket) {
    int rc = validate(h, d, o, N);
    if (rc) return rc;
    if (!ticket) return fail(h, ODE_E_INVALID, "null ticket pointer");
    if (N > 0 && (!u0 || !p || !tspan || !u_out || !nsaved || !retcode))
        return fail(h, ODE_E_INVALID, "null input or output buffer");
    if (o->nsave > 0 && !saveat) return fail(h, ODE_E_INVALID, "nsave > 0 but saveat is null");
    auto r = std::make_shared<Request>();
    r->d = *d;
    r->o = *o;
    r->N = N;
    const size_t n = (size_t)d->n_states, np = (size_t)d->n_params;
    r->u0.assign(u0, u0 + n * N);
    r->p.assign(p, p + np * N);
    r->tspan.assign(tspan, tspan + 2 * N);
    if (o->nsave > 0) r->saveat.assign(saveat, saveat + (size_t)o->nsave * (o->saveat_per_traj ? (size_t)N : 1));
    if (npt) r->npt.assign(npt, npt + N);
    r->t_out = t_out;
    r->u_out = u_out;
    r->nsaved = nsaved;
    r->retcode = retcode;
    r->stats = stats;
    r->bytes = request_bytes(*r);
    std::unique_lock<std::mutex> lk(h->mu);
    CUDA_TRY(h, cudaSetDevice(h->device));
    rc = ensure_worker(h);
    if (rc) return rc;
    r->ticket = h->next_ticket++;
    h->tickets[r->ticket] = r;
    h->pending.push_back(r);
    h->n_submitted++;
    *ticket = r->ticket;
    h->cv.notify_all();
    return ODE_OK;
}

int ode_poll(ode_handle* h, uint64_t ticket, int32_t* done) {
    if (!h || !done) return fail(h, ODE_E_INVALID, "null handle or output");
    std::unique_lock<std::mutex> lk(h->mu);
    auto it = h->tickets.find(ticket);
    if (it == h->tickets.end()) return fail(h, ODE_E_NOTFOUND, "unknown ticket");
    *done = it->second->state == 2;
    if (*done) {
        int st = it->second->status;
        h->tickets.erase(it);
        return st;
    }
    return ODE_OK;
}

int ode_wait(ode_handle* h, uint64_t ticket, double timeout_s) {
    if (!h) return fail(h, ODE_E_INVALID, "null handle");
    std::unique_lock<std::mutex> lk(h->mu);
    auto it = h->tickets.find(ticket);
    if (it == h->tickets.end()) return fail(h, ODE_E_NOTFOUND, "unknown ticket");
    auto r = it->second;
    auto pred = [&] { return r->state == 2; };
    if (timeout_s < 0) {
        h->cv.wait(lk, pred);
    } else if (!h->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) {
        return fail(h, ODE_E_TIMEOUT, "request not finished");
    }
    h->tickets.erase(ticket);
    return r->status;
}

int ode_serving_stats_get(ode_handle* h, ode_serving_stats* s) {
    if (!h || !s) return fail(h, ODE_E_INVALID, "null handle or output");
    std::unique_lock<std::mutex> lk(h->mu);
    s->submitted = h->n_submitted;
    s->admitted = h->n_admitted;
    s->completed = h->n_completed;
    s->rejected = h->n_rejected;
    s->queued = (int64_t)h->pending.size();
    s->running = (int64_t)h->running.size();
    s->hbm_in_use = (int64_t)h->hbm_in_use;
    s->hbm_budget = (int64_t)h->budget;
    s->slots = h->slots;
    s->reserved = 0;
    return ODE_OK;
}

int ode_set_serving_slots(ode_handle* h, int32_t slots) {
    if (!h || slots < 1 || slots > 64) return fail(h, ODE_E_INVALID, "slots must be in [1, 64]");
    std::unique_lock<std::mutex> lk(h->mu);
    if (h->worker_started) return fail(h, ODE_E_BUSY, "serving already started");
    h->slots = slots;
    return ODE_OK;
}

int ode_abort(ode_handle* h) {
    if (!h) return fail(h, ODE_E_INVALID, "null handle");
    __atomic_store_n(h->h_abort, 1, __ATOMIC_SEQ_CST);
    return ODE_OK;
}

int ode_kernel_launches(const ode_handle* h, int64_t* launches) {
    if (!h || !launches) return ODE_E_INVALID;
    *launches = h->launches.load();
    return ODE_OK;
}

int ode_last_kernel_ms(const ode_handle* h, double* ms) {
    if (!h || !ms) return ODE_E_INVALID;
    float f = 0;
    if (cudaEventElapsedTime(&f, h->main.ev0, h->main.ev1) == cudaSuccess) {
        *ms = f;
        return ODE_OK;
    }
    *ms = h->last_ms;
    return ODE_OK;
}

int ode_query_variants(int alg, int model, int precision, int n, int32_t* lanes, int32_t cap) {
    int k = 0;
    for (const auto& v : all_variants())
        if (v.alg == alg && v.model == model && v.prec == precision && v.n == n) {
            if (lanes && k < cap) lanes[k] = v.lanes;
            ++k;
        }
    return k;
}

}  // extern "C"

// ============================================================== allocation-free entry point
// For callers that must not allocate device memory: code running inside a
// framework whose caching allocator owns the GPU, callers under a strict
// memory budget, or hosts whose only device call surface is kernel launches
// and copies.  The scratch the bucketed persistent kernels need (work
// counters, per-size-class counts and offsets, the bucketed trajectory
// indices) lives in one file-scope device array instead of handle-owned
// cudaMalloc memory.
namespace {

// At most kNoAllocMaxTraj trajectories per call when per-trajectory sizes are
// given (the bucket index list); uniform-size calls only use the counters.
constexpr long long kNoAllocMaxTraj = 1LL << 20;
// [0, 8) work counters, [8, 16) class counts, [16, 24) class cursors,
// [32, 32 + kNoAllocMaxTraj) bucketed trajectory indices.  8 MiB + 256 B,
// held by every GPU that loads the library until the process exits.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[32 + kNoAllocMaxTraj];

std::mutex g_noalloc_mu;
unsigned long long* g_noalloc_ptr[64] = {};

// Device address of the scratch for the current device, resolved once per
// device (with that device current) and cached.
int noalloc_scratch(int dev, unsigned long long** out) {
    if (dev < 0 || dev >= 64) return fail(nullptr, ODE_E_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || ptr == nullptr)
            return fail(nullptr, ODE_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_noalloc_ptr[dev] = (unsigned long long*)ptr;
    }
    *out = g_noalloc_ptr[dev];
    return ODE_OK;
}

int noalloc_launch(const KernelVariant* v, EnsembleArgs a, unsigned long long* queue, int sm_count, cudaStream_t s) {
    if (a.count <= 0) return ODE_OK;
    const int block = 128;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, v->fn, block, 0);
    if (e != cudaSuccess) return fail(nullptr, ODE_E_CUDA, std::string("occupancy: ") + cudaGetErrorString(e));
    if (per_sm <= 0) per_sm = 1;
    long long want = (a.count * v->lanes + block - 1) / block;
    int grid = (int)std::min<long long>((long long)per_sm * sm_count, want);
    if (grid < 1) grid = 1;
    a.persistent = 1;
    a.queue = queue;
    v->launch(a, grid, block, 0, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(nullptr, ODE_E_CUDA, std::string("launch ") + v->name + ": " + cudaGetErrorString(e));
    return ODE_OK;
}

}  // namespace

extern "C" int ode_solve_ensemble_noalloc(const ode_problem_desc* d, const ode_options* o, int64_t N,
                                          const int32_t* npt_dev, const double* u0, const double* p,
                                          const double* tspan, const double* saveat, double* t_out,
                                          double* u_out, int32_t* nsaved, int32_t* retcode, ode_stats* stats,
                                          void* cuda_stream) {
    if (!d || !o) return fail(nullptr, ODE_E_INVALID, "null problem or options");
    if (N < 0) return fail(nullptr, ODE_E_INVALID, "negative trajectory count");
    if (npt_dev && N > kNoAllocMaxTraj) {
        char buf[160];
        std::snprintf(buf, sizeof buf,
                      "ode_solve_ensemble_noalloc: %lld trajectories with per-trajectory sizes exceed the "
                      "fixed scratch maximum of %lld",
                      (long long)N, (long long)kNoAllocMaxTraj);
        return fail(nullptr, ODE_E_INVALID, buf);
    }
    if (d->alg_id < ODE_TSIT5 || d->alg_id > ODE_RODAS5P ||
        (d->precision != ODE_PREC_FP64 && d->precision != ODE_PREC_MIXED) ||
        d->model_id < ODE_MODEL_LINEAR || d->model_id > ODE_MODEL_BRUSSELATOR_1D || d->n_states <= 0 ||
        d->n_params != model_nparams(d->model_id) || !(o->reltol > 0) || !(o->abstol >= 0) || o->nsave < 0)
        return fail(nullptr, ODE_E_INVALID, "invalid problem description or options");
    if (npt_dev && d->model_id != ODE_MODEL_DUFFING_CHAIN)
        return fail(nullptr, ODE_E_UNSUPPORTED, "per-trajectory sizes are supported for DUFFING_CHAIN");
    if (N == 0) return ODE_OK;
    int dev = 0, sm_count = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return fail(nullptr, ODE_E_CUDA, std::string("device query: ") + cudaGetErrorString(e));
    unsigned long long* scratch = nullptr;
    int rc = noalloc_scratch(dev, &scratch);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)cuda_stream;

    EnsembleArgs a;
    std::memset(&a, 0, sizeof(a));
    a.N = N;
    a.count = N;
    a.nmax = d->n_states;
    a.u0 = u0;
    a.p = p;
    a.tspan = tspan;
    a.saveat = saveat;
    a.nsave = o->nsave;
    a.saveat_per_traj = o->saveat_per_traj;
    a.nsave_cap = o->nsave + 2;
    a.t_out = t_out;
    a.u_out = u_out;
    a.nsaved = nsaved;
    a.retcode = retcode;
    a.stats = (OdeStatsDev*)stats;
    a.reltol = o->reltol;
    a.abstol = o->abstol;
    a.dtmax = o->dtmax;
    a.dtmin = o->dtmin;
    a.dt = o->dt;
    a.maxiters = o->maxiters > 0 ? o->maxiters : 1000000;
    a.save_start = o->save_start;
    a.save_end = o->save_end;
    a.save_end_user = o->save_end_user;
    a.saveat_given = o->nsave > 0;
    a.saveat_scalar = o->saveat_scalar;
    a.qmax_first_step = o->qmax_first_step;
    a.qmax = o->qmax;
    a.ir_sweeps = o->ir_sweeps < 0 ? 0 : o->ir_sweeps;
    a.abort_flag = nullptr;

    // Counters must start at zero on every call (the array keeps the last call's contents).
    e = cudaMemsetAsync(scratch, 0, 32 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return fail(nullptr, ODE_E_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    if (npt_dev == nullptr) {
        const KernelVariant* v = find_variant(d->alg_id, d->model_id, d->precision, d->n_states, o->lanes_per_traj);
        if (!v) return fail(nullptr, ODE_E_UNSUPPORTED, "no compiled kernel for this problem");
        return noalloc_launch(v, a, scratch, sm_count, s);
    }
    long long* order = (long long*)(scratch + 32);
    const int gb = (int)((N + 255) / 256);
    bucket_count<<<gb, 256, 0, s>>>(npt_dev, N, scratch + 8);
    unsigned long long hc[8] = {0};
    e = cudaMemcpyAsync(hc, scratch + 8, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(nullptr, ODE_E_CUDA, std::string("bucket counts: ") + cudaGetErrorString(e));
    unsigned long long off[8] = {0};
    unsigned long long acc = 0;
    for (int k = 0; k < 5; ++k) { off[k] = acc; acc += hc[k]; }
    e = cudaMemcpyAsync(scratch + 16, off, 5 * sizeof(unsigned long long), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(nullptr, ODE_E_CUDA, std::string("bucket offsets: ") + cudaGetErrorString(e));
    bucket_scatter<<<gb, 256, 0, s>>>(npt_dev, N, scratch + 16, order);
    for (int k = 0; k < 5; ++k) {
        if (hc[k] == 0) continue;
        const KernelVariant* v = find_variant(d->alg_id, d->model_id, d->precision, kClassN[k], 0);
        if (!v) return fail(nullptr, ODE_E_UNSUPPORTED, "no compiled kernel for a Duffing size class");
        EnsembleArgs ac = a;
        ac.order = order + off[k];
        ac.count = (long long)hc[k];
        rc = noalloc_launch(v, ac, scratch + k, sm_count, s);
        if (rc) return rc;
    }
    return ODE_OK;
}
