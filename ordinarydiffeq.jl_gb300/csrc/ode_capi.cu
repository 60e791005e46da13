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
#include "rtc_models.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
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
        t = rodas_group_variants(&n);
        out.insert(out.end(), t, t + n);
        t = ros23_variants(&n);
        out.insert(out.end(), t, t + n);
        t = ros23_group_variants(&n);
        out.insert(out.end(), t, t + n);
        t = auto_variants(&n);
        out.insert(out.end(), t, t + n);
        return out;
    }();
    return v;
}

int model_nparams(int model) {
    int np = 0;
    if (model >= ODE_MODEL_USER_BASE) return rtc_lookup(model, nullptr, &np, nullptr) ? np : -1;
    return (model == ODE_MODEL_LINEAR || model == ODE_MODEL_VANDERPOL) ? 1 : model == ODE_MODEL_FORCED_DUFFING ? 5 : 3;
}
// models with a registered callback (continuous: the ball; discrete: the dosing model)
bool model_has_event(int model) {
    int flags = 0;
    if (model >= ODE_MODEL_USER_BASE)
        return rtc_lookup(model, nullptr, nullptr, &flags) &&
               (flags & (ODE_MODEL_CONTINUOUS_CALLBACK | ODE_MODEL_VECTOR_CALLBACK | ODE_MODEL_DISCRETE_CALLBACK));
    return model == ODE_MODEL_BOUNCING_BALL || model == ODE_MODEL_PK_ONE_COMPARTMENT;
}

// Default lanes per trajectory: one lane for tiny systems (registers hold the
// whole state and stage set); explicit methods 4 states per lane so the Vern7
// stage set stays in registers without spilling, mixed Vern7 2 (a smaller
// per-lane step: 1.2-1.5x faster measured); Rodas5P above 8 states one lane
// per 2 states (W in shared memory, rows spread over the group).
bool is_rosenbrock(int alg) { return alg == ODE_RODAS5P || alg == ODE_ROSENBROCK23; }

int default_lanes(int alg, int n, int prec) {
    if (alg == ODE_VERN7 && prec == ODE_PREC_MIXED && n >= 4 && n % 2 == 0) return std::min(32, n / 2);
    if (n <= 4 || (n <= 8 && is_rosenbrock(alg))) return 1;
    if (is_rosenbrock(alg)) return std::min(32, n / 2);
    return std::min(32, n / 4);
}

const KernelVariant* find_variant(int alg, int model, int prec, int n, int lanes) {
    const KernelVariant* best = nullptr;
    for (const auto& v : all_variants()) {
        if (v.alg != alg || v.model != model || v.prec != prec || v.n != n) continue;
        if (lanes > 0 && v.lanes != lanes) continue;
        if (!best) best = &v;
        if (lanes <= 0 && v.lanes == default_lanes(alg, n, prec)) best = &v;
    }
    return best;
}

// The kernel of a uniform-size problem: a compiled-in variant, or the run-time
// compiled kernel of a registered model (compiled on its first use).  nullptr
// with *rc and *why set when there is none.
const KernelVariant* variant_for(const ode_problem_desc* d, int lanes, int* rc, std::string* why) {
    *rc = ODE_OK;
    if (d->model_id >= ODE_MODEL_USER_BASE) {
        if (lanes > 1) {
            *rc = ODE_E_UNSUPPORTED;
            *why = "registered models run one lane per trajectory";
            return nullptr;
        }
        return rtc_variant(d->alg_id, d->model_id, d->precision, rc, why);
    }
    const KernelVariant* v = find_variant(d->alg_id, d->model_id, d->precision, d->n_states, lanes);
    if (!v) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "no compiled kernel for alg %d model %d precision %d n %d lanes %d",
                      d->alg_id, d->model_id, d->precision, d->n_states, lanes);
        *rc = ODE_E_UNSUPPORTED;
        *why = buf;
    }
    return v;
}

// Launch one ensemble kernel: through its typed launcher, or (a registered
// model's run-time compiled kernel) through cudaLaunchKernel.
// The kernel a launch runs: the forward-only form when every span runs forward
// and the variant has one.
const void* kernel_fn(const KernelVariant* v, const EnsembleArgs& a) {
    return a.forward_only && v->fwd_fn ? v->fwd_fn : v->fn;
}

void launch_any(const KernelVariant* v, const EnsembleArgs& a, int grid, int block, size_t smem, cudaStream_t s) {
    if (a.forward_only && v->fwd_launch) {
        v->fwd_launch(a, grid, block, smem, s);
        return;
    }
    if (v->launch) {
        v->launch(a, grid, block, smem, s);
        return;
    }
    void* args[] = {const_cast<EnsembleArgs*>(&a)};
    cudaLaunchKernel(v->fn, dim3(grid), dim3(block), args, smem, s);
}

// Every span of a host tspan array runs forward (tf >= t0; NaN is not).
bool all_forward(const double* tspan, int64_t N) {
    for (int64_t j = 0; j < N; ++j)
        if (!(tspan[N + j] >= tspan[j])) return false;
    return true;
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
    // the last solve captured as a CUDA graph, replayed while its key matches
    cudaGraphExec_t graph = nullptr;
    std::vector<unsigned char> graph_key;
    long long graph_kernels = 0;
};

struct Request;
struct Batch;

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
    DevBuf b_k, b_tq, b_out;                 // dense output and its evaluation
    DevBuf b_tstops;                         // the host API's tstops, sorted
    DevBuf b_idx;                            // the host API's save_idxs
    DevBuf b_atol, b_rtol;                   // the host API's per-state tolerances
    // copy streams and events of the chunked host-API pipeline
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    cudaEvent_t pipe_in[4] = {}, pipe_done[4] = {};
    std::mutex api_mu;
    // serving
    std::mutex mu;
    std::condition_variable cv;
    std::list<std::shared_ptr<Request>> pending;
    std::vector<std::shared_ptr<Batch>> running;
    std::map<uint64_t, std::shared_ptr<Request>> tickets;
    std::thread worker;
    bool stop = false;
    bool worker_started = false;
    int slots = 8;
    uint64_t next_ticket = 1;
    size_t hbm_in_use = 0;
    long long n_submitted = 0, n_admitted = 0, n_completed = 0, n_rejected = 0, n_batches = 0;
    size_t max_queued = 0;                   // ode_submit answers ODE_E_BUSY past this many queued (0: no limit)
    std::vector<Ctx> slot_ctx;
    std::vector<int> slot_busy;
    std::vector<void*> slot_pinned;          // per-slot pinned staging (grow only)
    std::vector<size_t> slot_pinned_cap;
    std::vector<cudaEvent_t> slot_ev;        // end of the slot's current request
    std::deque<uint64_t> completed;          // tickets in completion order
    // autotuned launch shape per (alg, model, precision, n)
    struct Tuned { int lanes, block, scheduler; double ms; };
    std::map<std::tuple<int, int, int, int>, Tuned> tuned;
    std::mutex tune_mu;
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

// Checks of a problem and its options that need no handle, shared by every
// entry point (the allocation-free one included), so that each rejects the same
// input with the same status.  Returns ODE_OK or the status, with the reason in *why.
int check_problem(const ode_problem_desc* d, const ode_options* o, int64_t N, const char** why) {
    auto bad = [&](int code, const char* msg) { *why = msg; return code; };
    if (!d || !o) return bad(ODE_E_INVALID, "null problem or options");
    if (N < 0) return bad(ODE_E_INVALID, "negative trajectory count");
    if (d->alg_id < ODE_TSIT5 || d->alg_id >= kNumAlgs) return bad(ODE_E_INVALID, "unknown alg_id");
    if (d->model_id >= ODE_MODEL_USER_BASE) {
        int n = 0;
        if (!rtc_lookup(d->model_id, &n, nullptr, nullptr)) return bad(ODE_E_INVALID, "unknown model_id");
        if (d->n_states != n) return bad(ODE_E_INVALID, "n_states does not match the registered model");
    } else if (d->model_id < ODE_MODEL_LINEAR || d->model_id > ODE_MODEL_FORCED_DUFFING) {
        return bad(ODE_E_INVALID, "unknown model_id");
    }
    if (d->precision != ODE_PREC_FP64 && d->precision != ODE_PREC_MIXED)
        return bad(ODE_E_INVALID, "unknown precision");
    if (d->n_states <= 0) return bad(ODE_E_INVALID, "n_states must be positive");
    if (d->n_params != model_nparams(d->model_id)) return bad(ODE_E_INVALID, "n_params does not match the model");
    if ((d->model_id == ODE_MODEL_LORENZ || d->model_id == ODE_MODEL_ROBERTSON) && d->n_states != 3)
        return bad(ODE_E_INVALID, "this model has 3 states");
    if ((d->model_id == ODE_MODEL_BOUNCING_BALL || d->model_id == ODE_MODEL_VANDERPOL ||
         d->model_id == ODE_MODEL_PK_ONE_COMPARTMENT || d->model_id == ODE_MODEL_FORCED_DUFFING) &&
        d->n_states != 2)
        return bad(ODE_E_INVALID, "this model has 2 states");
    if (o->callback && !model_has_event(d->model_id))
        return bad(ODE_E_UNSUPPORTED, "the model has no registered callback");
    if (o->callback && (o->interp_points < 0 || o->max_events < 0))
        return bad(ODE_E_INVALID, "interp_points and max_events must be >= 0");
    if (!(o->reltol > 0) || !(o->abstol >= 0)) return bad(ODE_E_INVALID, "tolerances must be positive");
    if (o->nsave < 0) return bad(ODE_E_INVALID, "negative nsave");
    if (o->save_everystep && o->max_step_saves <= 0)
        return bad(ODE_E_INVALID, "save_everystep needs max_step_saves > 0");
    if (o->ntstops < 0 || (o->ntstops > 0 && !o->tstops))
        return bad(ODE_E_INVALID, "ntstops < 0, or tstops is null");
    if (o->max_jac_age < 0) return bad(ODE_E_INVALID, "max_jac_age must be >= 0");
    if (o->isoutofdomain < 0 || o->isoutofdomain > 1)
        return bad(ODE_E_INVALID, "isoutofdomain must be 0 (none) or 1 (any state < 0)");
    if (o->nsave_idxs < 0 || (o->nsave_idxs > 0 && !o->save_idxs))
        return bad(ODE_E_INVALID, "nsave_idxs < 0, or save_idxs is null");
    if (o->controller_given) {
        const double f[] = {o->beta1, o->beta2, o->qoldinit, o->qmin, o->gamma, o->qsteady_min, o->qsteady_max};
        for (double v : f)
            if (std::isinf(v)) return bad(ODE_E_INVALID, "controller knobs must be finite (NaN: the default)");
        if (o->qmin <= 0 || o->gamma <= 0 || o->qoldinit <= 0)
            return bad(ODE_E_INVALID, "controller qmin, gamma and qoldinit must be > 0");
    }
    if (!o->adaptive && (std::isnan(o->dt) || std::isinf(o->dt) || (o->dt == 0 && o->ntstops == 0)))
        return bad(ODE_E_INVALID, "fixed steps (adaptive = 0) need a finite dt or tstops");
    // the kept J lives beside W in registers; the shared-memory LU (16-64 states)
    // forms W in place of J
    if (d->alg_id == ODE_ROSENBROCK23 && o->max_jac_age > 1 && d->n_states > 8)
        return bad(ODE_E_UNSUPPORTED, "Rosenbrock23 Jacobian reuse (max_jac_age > 1) needs n_states <= 8");
    if (o->jac_reuse_gamma_tol != o->jac_reuse_gamma_tol)
        return bad(ODE_E_INVALID, "jac_reuse_gamma_tol is NaN");
    return ODE_OK;
}

int validate(ode_handle* h, const ode_problem_desc* d, const ode_options* o, int64_t N) {
    if (!h) return fail(h, ODE_E_INVALID, "null handle");
    const char* why = "";
    const int rc = check_problem(d, o, N, &why);
    return rc ? fail(h, rc, why) : ODE_OK;
}

// The host entry points take tstops in host memory, in any order: checked for
// NaN here, then sorted (the kernels walk them in ascending order).
int check_host_tstops(ode_handle* h, const ode_options* o) {
    for (int32_t i = 0; i < o->ntstops; ++i)
        if (o->tstops[i] != o->tstops[i]) return fail(h, ODE_E_INVALID, "NaN in tstops");
    return ODE_OK;
}

// ... and their save_idxs in host memory: each a state of the problem.
int check_host_save_idxs(ode_handle* h, const ode_problem_desc* d, const ode_options* o) {
    for (int32_t r = 0; r < o->nsave_idxs; ++r)
        if (o->save_idxs[r] < 0 || o->save_idxs[r] >= d->n_states)
            return fail(h, ODE_E_INVALID, "save_idxs entry outside [0, n_states)");
    return ODE_OK;
}

// Per-state tolerances given in host memory: every entry finite, abstol >= 0, reltol > 0.
int check_host_tolvec(ode_handle* h, const ode_problem_desc* d, const ode_options* o) {
    for (int32_t i = 0; i < d->n_states; ++i) {
        if (o->abstol_vec && !(o->abstol_vec[i] >= 0 && std::isfinite(o->abstol_vec[i])))
            return fail(h, ODE_E_INVALID, "abstol_vec entries must be finite and >= 0");
        if (o->reltol_vec && !(o->reltol_vec[i] > 0 && std::isfinite(o->reltol_vec[i])))
            return fail(h, ODE_E_INVALID, "reltol_vec entries must be finite and > 0");
    }
    return ODE_OK;
}

// Output rows per save: the save_idxs, else every state.
size_t out_rows(const ode_problem_desc* d, const ode_options* o) {
    return o->nsave_idxs > 0 ? (size_t)o->nsave_idxs : (size_t)d->n_states;
}

std::vector<double> sorted_tstops(const ode_options* o) {
    std::vector<double> v;
    if (o->ntstops > 0) v.assign(o->tstops, o->tstops + o->ntstops);
    std::sort(v.begin(), v.end());
    return v;
}

// Copy the sorted tstops into the handle's buffer on stream s (synchronously:
// they are a few bytes) and return in ot the options with tstops pointing
// there, the form the launch code takes.
int stage_tstops(ode_handle* h, const ode_options* o, cudaStream_t s, ode_options* ot) {
    *ot = *o;
    ot->tstops = nullptr;
    const std::vector<double> v = sorted_tstops(o);
    ot->ntstops = (int32_t)v.size();
    int rc = ODE_OK;
    if (!v.empty()) {
        if ((rc = grow(h, h->b_tstops, v.size() * 8))) return rc;
        CUDA_TRY(h, cudaMemcpyAsync(h->b_tstops.p, v.data(), v.size() * 8, cudaMemcpyHostToDevice, s));
        ot->tstops = (const double*)h->b_tstops.p;
    }
    if (o->nsave_idxs > 0) {   // the save_idxs too, as given
        if ((rc = grow(h, h->b_idx, (size_t)o->nsave_idxs * 4))) return rc;
        CUDA_TRY(h, cudaMemcpyAsync(h->b_idx.p, o->save_idxs, (size_t)o->nsave_idxs * 4, cudaMemcpyHostToDevice, s));
        ot->save_idxs = (const int32_t*)h->b_idx.p;
    }
    CUDA_TRY(h, cudaStreamSynchronize(s));
    return ODE_OK;
}

// The host API's per-state tolerances into the handle's buffers (ot's pointers
// still the caller's host arrays), synchronously: n doubles each.
int stage_tolvec(ode_handle* h, const ode_problem_desc* d, cudaStream_t s, ode_options* ot) {
    int rc = ODE_OK;
    const size_t bytes = (size_t)d->n_states * 8;
    if (ot->abstol_vec) {
        if ((rc = grow(h, h->b_atol, bytes))) return rc;
        CUDA_TRY(h, cudaMemcpyAsync(h->b_atol.p, ot->abstol_vec, bytes, cudaMemcpyHostToDevice, s));
        ot->abstol_vec = (const double*)h->b_atol.p;
    }
    if (ot->reltol_vec) {
        if ((rc = grow(h, h->b_rtol, bytes))) return rc;
        CUDA_TRY(h, cudaMemcpyAsync(h->b_rtol.p, ot->reltol_vec, bytes, cudaMemcpyHostToDevice, s));
        ot->reltol_vec = (const double*)h->b_rtol.p;
    }
    if (ot->abstol_vec || ot->reltol_vec) CUDA_TRY(h, cudaStreamSynchronize(s));
    return ODE_OK;
}

// Output slots per trajectory: the saveat points (or the kept step saves)
// plus the start and end saves.
size_t save_cap(const ode_options* o) {
    return (size_t)o->nsave + (o->save_everystep ? (size_t)o->max_step_saves : 0) + 2 +
           (o->callback ? 2 * (size_t)o->max_events : 0);
}

// The PI controller of each method of alg (slot 1: the composite's stiff method):
// the method's defaults (alg_utils.jl: beta2 = 2/(5 order), beta1 = 7/(10 order),
// qmin 1/5, qmax 10, qmax_first_step 10^4, gamma 9/10, qsteady_min 1, qsteady_max
// 6/5 for the adaptive implicit family else 1, qoldinit 10^-4), then the caller's
// knobs, in FP64 and FP32 for the two precisions' controllers.
void resolve_controller(EnsembleArgs& a, int alg_id, const ode_options* o) {
    struct Method { int order; bool implicit; };
    Method m[2] = {{5, false}, {5, false}};
    switch (alg_id) {
        case ODE_VERN7: m[0] = {7, false}; break;
        case ODE_RODAS5P: m[0] = {5, true}; break;
        case ODE_ROSENBROCK23: m[0] = {2, true}; break;
        case ODE_AUTOTSIT5_ROSENBROCK23: m[1] = {2, true}; break;   // Tsit5, then Rosenbrock23
        default: break;
    }
    for (int s = 0; s < 2; ++s) {
        double v[KNCTRL];
        v[KB2] = 2.0 / (5.0 * m[s].order);
        v[KB1] = 7.0 / (10.0 * m[s].order);
        double qmin = 0.2, gamma = 0.9;
        v[KQSMIN] = 1.0;
        v[KQSMAX] = m[s].implicit ? 1.2 : 1.0;
        v[KQOLD] = 1e-4;
        if (o->controller_given) {   // each knob that is not NaN
            auto set = [](double& f, double x) { if (!std::isnan(x)) f = x; };
            set(v[KB1], o->beta1);
            set(v[KB2], o->beta2);
            set(v[KQOLD], o->qoldinit);
            set(qmin, o->qmin);
            set(gamma, o->gamma);
            set(v[KQSMIN], o->qsteady_min);
            set(v[KQSMAX], o->qsteady_max);
        }
        v[KQMININV] = 1.0 / qmin;
        v[KQMIN] = qmin;
        v[KGAM] = gamma;
        v[KIQMAX] = 1.0 / (o->qmax > 0 ? o->qmax : 10.0);
        v[KIQMAXF] = 1.0 / (o->qmax_first_step > 0 ? o->qmax_first_step : 10000.0);
        for (int k = 0; k < KNCTRL; ++k) {
            a.kd[s][k] = v[k];
            a.kf[s][k] = (float)v[k];
        }
    }
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
    a.nsave_cap = (int)save_cap(o);
    a.save_everystep = o->save_everystep;
    a.callback = o->callback ? 1 : 0;
    a.interp_points = o->interp_points;
    a.tstops = o->ntstops > 0 ? o->tstops : nullptr;   // device memory, ascending, at this point
    a.ntstops = o->ntstops > 0 ? o->ntstops : 0;
    a.max_jac_age = o->max_jac_age;
    a.jac_reuse_gamma_tol = o->jac_reuse_gamma_tol < 0 ? 0.03 : o->jac_reuse_gamma_tol;
    a.adaptive = o->adaptive ? 1 : 0;
    a.forward_only = (o->forward_only && !o->force_dtmin && !o->isoutofdomain) ? 1 : 0;
    a.abstol_vec = o->abstol_vec;
    a.reltol_vec = o->reltol_vec;
    a.force_dtmin = o->force_dtmin ? 1 : 0;
    a.isoutofdomain = o->isoutofdomain;
    resolve_controller(a, d->alg_id, o);
    a.save_idxs = o->nsave_idxs > 0 ? o->save_idxs : nullptr;   // device memory at this point
    a.nsave_rows = o->nsave_idxs > 0 ? o->nsave_idxs : 0;
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

// Size class of a state count: 4, 8, 16, 32, 64 -> 0..4; -1 for any other.
__device__ __forceinline__ int size_class(int n) {
    return n == 4 ? 0 : n == 8 ? 1 : n == 16 ? 2 : n == 32 ? 3 : n == 64 ? 4 : -1;
}

// Bucket trajectories by state count on the device: a histogram, then a
// scatter of the indices into class order (class k at [offset[k],
// offset[k] + count[k])).  Atomics are aggregated per warp (one per class).
// Trajectories of any other size are not integrated: nsaved 0, retcode DEFAULT.
__global__ void bucket_count(const int32_t* npt, long long N, unsigned long long* counts) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int c = j < N ? size_class(npt[j]) : -2;
    if (c == -1) c = kNumClasses;
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k <= kNumClasses; ++k) {
        const unsigned m = __ballot_sync(0xffffffffu, c == k);
        if (m && lane == __ffs(m) - 1) atomicAdd(&counts[k], (unsigned long long)__popc(m));
    }
}
__global__ void bucket_scatter(const int32_t* npt, long long N, const unsigned long long* counts,
                               unsigned long long* cursor, unsigned long long* offsets, long long* order,
                               int32_t* nsaved, int32_t* retcode) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long off[kNumClasses];
    unsigned long long acc = 0;
#pragma unroll
    for (int k = 0; k < kNumClasses; ++k) { off[k] = acc; acc += counts[k]; }
    if (blockIdx.x == 0 && threadIdx.x < kNumClasses) offsets[threadIdx.x] = off[threadIdx.x];
    const int c = j < N ? size_class(npt[j]) : -2;
    if (c == -1) {
        nsaved[j] = 0;
        retcode[j] = ODE_RC_DEFAULT;
    }
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < kNumClasses; ++k) {
        const unsigned m = __ballot_sync(0xffffffffu, c == k);
        if (!m) continue;
        const int leader = __ffs(m) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(&cursor[k], (unsigned long long)__popc(m));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (c == k) order[off[k] + base + __popc(m & lt)] = j;
    }
}

// Device counters of one context: [0] the work queue of a uniform launch,
// then, for uneven ensembles, class counts (5 classes + invalid sizes), scatter
// cursors, per-class work counters, class offsets and the per-class queues of
// the one-kernel-per-class form.
constexpr int kCounters = 64;
constexpr int kOffCounts = 8, kOffCursor = 16, kOffNext = 24, kOffOffsets = 32, kOffClassQ = 40;

const FusedVariant* find_fused(int alg, int model, int prec) {
    static const std::vector<FusedVariant> all = [] {
        std::vector<FusedVariant> out;
        int n = 0;
        const FusedVariant* t = fused_tsit5_variants(&n);
        out.insert(out.end(), t, t + n);
        t = fused_vern7_variants(&n);
        out.insert(out.end(), t, t + n);
        return out;
    }();
    for (const auto& v : all)
        if (v.alg == alg && v.model == model && v.prec == prec) return &v;
    return nullptr;
}

// Count + scatter of an uneven ensemble into class order (device only).
void enqueue_count(const int32_t* npt_dev, long long N, unsigned long long* ctr, cudaStream_t s) {
    bucket_count<<<(int)((N + 255) / 256), 256, 0, s>>>(npt_dev, N, ctr + kOffCounts);
}
void enqueue_scatter(const int32_t* npt_dev, long long N, unsigned long long* ctr, long long* order,
                     int32_t* nsaved, int32_t* retcode, cudaStream_t s) {
    bucket_scatter<<<(int)((N + 255) / 256), 256, 0, s>>>(npt_dev, N, ctr + kOffCounts, ctr + kOffCursor,
                                                          ctr + kOffOffsets, order, nsaved, retcode);
}
void enqueue_bucketing(const int32_t* npt_dev, long long N, unsigned long long* ctr, long long* order,
                       int32_t* nsaved, int32_t* retcode, cudaStream_t s) {
    enqueue_count(npt_dev, N, ctr, s);
    enqueue_scatter(npt_dev, N, ctr, order, nsaved, retcode, s);
}

// The one-kernel-per-class form needs a compiled kernel for every size class
// present (hc: the class counts read back); a missing one fails the solve
// before the scatter, i.e. before anything is written to the outputs.
int class_kernels(ode_handle* h, const ode_problem_desc* d, const unsigned long long* hc,
                  const KernelVariant** vk) {
    for (int k = 0; k < kNumClasses; ++k) {
        vk[k] = nullptr;
        if (hc[k] == 0) continue;
        vk[k] = find_variant(d->alg_id, d->model_id, d->precision, kClassStates[k], 0);
        if (!vk[k]) {
            char buf[160];
            std::snprintf(buf, sizeof buf, "no compiled kernel for alg %d on the %d-state Duffing size class",
                          d->alg_id, kClassStates[k]);
            return fail(h, ODE_E_UNSUPPORTED, buf);
        }
    }
    return ODE_OK;
}

// Every size class in one persistent launch (grid = resident blocks x SMs).
cudaError_t launch_fused(const FusedVariant* fv, EnsembleArgs a, unsigned long long* ctr, int sm_count,
                         cudaStream_t s) {
    const int block = 128;
    int per_sm = 0;
    const bool fwd = a.forward_only && fv->fwd_fn;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fwd ? fv->fwd_fn : fv->fn, block, 0);
    if (e != cudaSuccess) return e;
    if (per_sm <= 0) per_sm = 1;
    long long want = (a.count * 16 + block - 1) / block;   // enough groups for the largest class
    int grid = (int)std::min<long long>((long long)per_sm * sm_count, std::max<long long>(want, 1));
    a.persistent = 1;
    a.refill_lanes = 16;   // measured best of 8, 16 and 32 on 1M uneven Duffing chains
    a.class_count = ctr + kOffCounts;
    a.class_offset = ctr + kOffOffsets;
    a.class_next = ctr + kOffNext;
    (fwd ? fv->fwd_launch : fv->launch)(a, grid, block, 0, s);
    return cudaGetLastError();
}
constexpr int kBlock = 128;

// Block size and dynamic shared memory of a launch.  Variants that keep W in
// shared memory default to one warp per block (finer occupancy steps).
cudaError_t launch_geometry(const KernelVariant* v, int block, int* block_out, size_t* smem_out) {
    if (v->lanes > 1 && block % 32 != 0) block = kBlock;
    if (block <= 0) block = v->smem_per_group > 0 ? 32 : kBlock;
    if (block > 128) block = 128;
    if (v->smem_per_group > 0) {   // shrink the block until its groups' W fit in one SM
        int dev = 0, max_optin = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e != cudaSuccess) return e;
        while (block > 32 && block > v->lanes && (size_t)(block / v->lanes) * v->smem_per_group > (size_t)max_optin)
            block /= 2;
    }
    const size_t smem = (size_t)(block / v->lanes) * (size_t)v->smem_per_group;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(v->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess && v->fwd_fn)
            e = cudaFuncSetAttribute(v->fwd_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    *block_out = block;
    *smem_out = smem;
    return cudaSuccess;
}

int launch_variant(ode_handle* h, const KernelVariant* v, EnsembleArgs a, int scheduler, int block,
                   unsigned long long* queue, cudaStream_t s) {
    if (a.count <= 0) return ODE_OK;
    size_t smem = 0;
    {
        cudaError_t e = launch_geometry(v, block, &block, &smem);
        if (e != cudaSuccess) return fail(h, ODE_E_CUDA, std::string("shared memory for ") + v->name + ": " + cudaGetErrorString(e));
    }
    long long groups = a.count;
    bool persistent = scheduler == 2;
    int grid;
    if (persistent) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel_fn(v, a), block, smem);
        if (per_sm <= 0) per_sm = 1;
        long long want = (groups * v->lanes + block - 1) / block;
        grid = (int)std::min<long long>((long long)per_sm * h->sm_count, want);
        if (grid < 1) grid = 1;
        CUDA_TRY(h, cudaMemsetAsync(queue, 0, sizeof(unsigned long long), s));
        a.queue = queue;
        a.persistent = 1;
        a.refill_lanes = 4;    // 100k van der Pol (AutoTsit5) FP64: 217 ms at 4 idle lanes, 215 at 2, 232 at 8, 276 at 16, 436 at 32
    } else {
        long long threads = groups * v->lanes;
        grid = (int)((threads + block - 1) / block);
        a.persistent = 0;
        a.refill_lanes = 32;   // nothing to refill: lanes leave together
    }
    launch_any(v, a, grid, block, smem, s);
    h->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(h, ODE_E_CUDA, std::string("launch ") + v->name + ": " + cudaGetErrorString(e));
    return ODE_OK;
}

int ctx_init(ode_handle* h, Ctx& c, cudaStream_t s) {
    if (s) c.stream = s;
    else CUDA_TRY(h, cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
    CUDA_TRY(h, cudaMalloc(&c.d_queue, kCounters * sizeof(unsigned long long)));
    CUDA_TRY(h, cudaMemset(c.d_queue, 0, kCounters * sizeof(unsigned long long)));
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
    if (c.graph) cudaGraphExecDestroy(c.graph);
    if (c.stream) cudaStreamDestroy(c.stream);
    c = Ctx();
}

// The kernels of one solve, chosen before anything is enqueued.
struct Plan {
    const KernelVariant* v = nullptr;   // uniform size
    const FusedVariant* fv = nullptr;   // uneven sizes, one launch over all classes
    int block = 0, scheduler = 0;
    bool per_class = false;             // uneven sizes without a fused kernel
};

int make_plan(ode_handle* h, const ode_problem_desc* d, const ode_options* o, const int32_t* npt_dev, Plan* pl) {
    *pl = Plan();
    pl->scheduler = o->scheduler;
    pl->block = o->block_size;
    if (npt_dev == nullptr) {
        int lanes = o->lanes_per_traj;
        if (lanes <= 0 && pl->block <= 0 && pl->scheduler == 0) {   // shape chosen by ode_autotune, if any
            std::lock_guard<std::mutex> tl(h->tune_mu);
            auto it = h->tuned.find(std::make_tuple(d->alg_id, d->model_id, d->precision, d->n_states));
            if (it != h->tuned.end()) {
                lanes = it->second.lanes;
                pl->block = it->second.block;
                pl->scheduler = it->second.scheduler;
            }
        }
        int rc = ODE_OK;
        std::string why;
        pl->v = variant_for(d, lanes, &rc, &why);
        if (!pl->v) return fail(h, rc, why);
        // auto: the persistent queue for the shared-memory kernels (measured 13%
        // faster on the 64-state Brusselator: its many short waves leave tails)
        // and for AutoTsit5 (trajectories that turn stiff take ~100x the steps of
        // the others, and a finished lane refills: 498 -> 295 ms on 100k van der
        // Pol oscillators), one group per trajectory otherwise
        if (pl->scheduler == 0)
            pl->scheduler = (pl->v->smem_per_group > 0 || d->alg_id == ODE_AUTOTSIT5_ROSENBROCK23) ? 2 : 1;
        return ODE_OK;
    }
    if (d->model_id != ODE_MODEL_DUFFING_CHAIN)
        return fail(h, ODE_E_UNSUPPORTED, "per-trajectory sizes are supported for DUFFING_CHAIN");
    pl->fv = o->lanes_per_traj <= 0 ? find_fused(d->alg_id, d->model_id, d->precision) : nullptr;
    pl->per_class = pl->fv == nullptr;
    if (pl->scheduler == 0) pl->scheduler = 2;
    return ODE_OK;
}

// Enqueue a uniform or one-launch uneven solve (device work only, no host
// synchronisation: capturable in a CUDA graph).
int enqueue_plan(ode_handle* h, Ctx& c, const Plan& pl, EnsembleArgs a, const int32_t* npt_dev, cudaStream_t s) {
    if (pl.v) return launch_variant(h, pl.v, a, pl.scheduler, pl.block, c.d_queue, s);
    unsigned long long* ctr = c.d_queue;
    CUDA_TRY(h, cudaMemsetAsync(ctr + kOffCounts, 0, (kCounters - kOffCounts) * sizeof(unsigned long long), s));
    enqueue_bucketing(npt_dev, a.count, ctr, c.d_order, a.nsaved, a.retcode, s);
    h->launches += 2;
    a.order = c.d_order;
    cudaError_t e = launch_fused(pl.fv, a, ctr, h->sm_count, s);
    if (e != cudaSuccess) return fail(h, ODE_E_CUDA, std::string("launch ") + pl.fv->name + ": " + cudaGetErrorString(e));
    h->launches++;
    return ODE_OK;
}

// Uneven sizes without a fused kernel: one persistent kernel per size class on
// the class streams (the counts are read back to size the launches and to check
// that every class present has a kernel before anything is written).
int run_per_class(ode_handle* h, Ctx& c, const ode_problem_desc* d, const ode_options* o, const Plan& pl,
                  EnsembleArgs a, const int32_t* npt_dev, cudaStream_t s) {
    unsigned long long* ctr = c.d_queue;
    CUDA_TRY(h, cudaMemsetAsync(ctr + kOffCounts, 0, (kCounters - kOffCounts) * sizeof(unsigned long long), s));
    enqueue_count(npt_dev, a.count, ctr, s);
    h->launches += 1;
    unsigned long long hc[kNumClasses + 1] = {0};
    CUDA_TRY(h, cudaMemcpyAsync(hc, ctr + kOffCounts, sizeof(hc), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(h, cudaStreamSynchronize(s));
    const KernelVariant* vk[kNumClasses];
    int rc = class_kernels(h, d, hc, vk);
    if (rc) return rc;
    enqueue_scatter(npt_dev, a.count, ctr, c.d_order, a.nsaved, a.retcode, s);
    h->launches += 1;
    unsigned long long off[kNumClasses];
    unsigned long long acc = 0;
    for (int k = 0; k < kNumClasses; ++k) { off[k] = acc; acc += hc[k]; }
    CUDA_TRY(h, cudaEventRecord(c.ev0, s));
    for (int k = 0; k < kNumClasses; ++k) {
        if (hc[k] == 0) continue;
        CUDA_TRY(h, cudaStreamWaitEvent(c.class_streams[k], c.ev0, 0));
        EnsembleArgs ac = a;
        ac.order = c.d_order + off[k];
        ac.count = (long long)hc[k];
        rc = launch_variant(h, vk[k], ac, pl.scheduler, o->block_size, ctr + kOffClassQ + k, c.class_streams[k]);
        if (rc) return rc;
        CUDA_TRY(h, cudaEventRecord(c.class_events[k], c.class_streams[k]));
        CUDA_TRY(h, cudaStreamWaitEvent(s, c.class_events[k], 0));
    }
    CUDA_TRY(h, cudaEventRecord(c.ev1, s));
    return ODE_OK;
}

// Enqueue the whole ensemble on stream s using the scratch of ctx c.  All
// pointers are device pointers.  With `graph`, a solve whose arguments,
// kernels and stream equal the previous one of this context replays that
// solve's CUDA graph (memsets, bucketing and integrator launches as one
// graph launch); a new solve is captured and instantiated once.
int run_ensemble(ode_handle* h, Ctx& c, const ode_problem_desc* d, const ode_options* o, int64_t N,
                 const int32_t* npt_dev, const double* u0, const double* p, const double* tspan,
                 const double* saveat, double* t_out, double* u_out, int32_t* nsaved, int32_t* retcode,
                 OdeStatsDev* stats, cudaStream_t s, bool graph = false, int64_t stride = 0, bool timing = true,
                 double* k_out = nullptr, const double* reltol_traj = nullptr, const double* abstol_traj = nullptr) {
    EnsembleArgs a = make_args(h, d, o, N, u0, p, tspan, saveat, t_out, u_out, nsaved, retcode, stats);
    a.k_out = k_out;
    a.reltol_traj = reltol_traj;
    a.abstol_traj = abstol_traj;
    if (stride > 0) a.N = stride;   // a slice of a larger ensemble: N trajectories, arrays of row length stride
    if (N == 0) return ODE_OK;
    Plan pl;
    int rc = make_plan(h, d, o, npt_dev, &pl);
    if (rc) return rc;
    if (npt_dev && (size_t)N > c.order_cap) {
        if (c.d_order) cudaFree(c.d_order);
        c.d_order = nullptr;
        c.order_cap = 0;
        CUDA_TRY(h, cudaMalloc(&c.d_order, sizeof(long long) * (size_t)N));
        c.order_cap = (size_t)N;
    }
    if (pl.per_class) return run_per_class(h, c, d, o, pl, a, npt_dev, s);
    if (!graph || s == nullptr) {
        if (timing) CUDA_TRY(h, cudaEventRecord(c.ev0, s));
        rc = enqueue_plan(h, c, pl, a, npt_dev, s);
        if (rc) return rc;
        if (timing) CUDA_TRY(h, cudaEventRecord(c.ev1, s));
        return ODE_OK;
    }
    struct Key {
        EnsembleArgs a;
        const void* kernel;
        const int32_t* npt;
        cudaStream_t s;
        int block, scheduler;
    } key;
    std::memset(&key, 0, sizeof(key));
    key.a = a;
    key.kernel = pl.v ? (const void*)pl.v : (const void*)pl.fv;
    key.npt = npt_dev;
    key.s = s;
    key.block = pl.block;
    key.scheduler = pl.scheduler;
    const unsigned char* kb = reinterpret_cast<const unsigned char*>(&key);
    const bool hit = c.graph && c.graph_key.size() == sizeof(key) && std::memcmp(c.graph_key.data(), kb, sizeof(key)) == 0;
    if (!hit) {
        if (c.graph) cudaGraphExecDestroy(c.graph);
        c.graph = nullptr;
        c.graph_key.clear();
        const long long before = h->launches.load();
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            rc = enqueue_plan(h, c, pl, a, npt_dev, s);
            e = cudaStreamEndCapture(s, &g);
        }
        const long long kernels = h->launches.load() - before;
        h->launches -= kernels;   // captured, not launched yet
        cudaGraphExec_t ex = nullptr;
        if (rc == ODE_OK && e == cudaSuccess && g) e = cudaGraphInstantiate(&ex, g, 0);
        if (g) cudaGraphDestroy(g);
        if (rc != ODE_OK || e != cudaSuccess || !ex) {   // not capturable here: enqueue directly
            if (ex) cudaGraphExecDestroy(ex);
            cudaGetLastError();
            CUDA_TRY(h, cudaEventRecord(c.ev0, s));
            rc = enqueue_plan(h, c, pl, a, npt_dev, s);
            if (rc) return rc;
            CUDA_TRY(h, cudaEventRecord(c.ev1, s));
            return ODE_OK;
        }
        c.graph = ex;
        c.graph_key.assign(kb, kb + sizeof(key));
        c.graph_kernels = kernels;
    }
    CUDA_TRY(h, cudaEventRecord(c.ev0, s));
    CUDA_TRY(h, cudaGraphLaunch(c.graph, s));
    h->launches += c.graph_kernels;
    CUDA_TRY(h, cudaEventRecord(c.ev1, s));
    return ODE_OK;
}


// Device address of a page-locked host buffer (mapped into the device's
// address space), or nullptr for ordinary pageable memory.  On GB300 the GPU
// reaches page-locked Grace memory over NVLink-C2C, so kernels can read their
// inputs and write their saves there directly.
template <class T> T* mapped_ptr(T* ptr) {
    if (!ptr) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || at.devicePointer == nullptr) return nullptr;
    return (T*)at.devicePointer;
}

// Large host-buffer solves run as a pipeline of kPipeChunks trajectory slices:
// slice k+1's inputs go in on one copy stream while slice k integrates and
// slice k-1's outputs come back on another, so the transfers hide behind the
// kernels.  Row-major SoA arrays make each slice a pitched 2-D copy.
// Slices run one after another, so each pays a tail; the pipeline pays off
// only where the transfers are long next to the compute, i.e. for many bytes
// per trajectory (measured: 1M uneven Duffing chains, 9.2 KB each, 1.98 ->
// 3.79 M traj/s end to end; Robertson, 0.7 KB, and the 64-state Brusselator,
// 6 KB, lose 10-30% when sliced).
constexpr int64_t kPipeMin = 32768;
constexpr size_t kPipeMinBytesPerTraj = 8192;
constexpr int kPipeChunks = 4;

int solve_chunked(ode_handle* h, const ode_problem_desc* d, const ode_options* o, int64_t N, const int32_t* npt,
                  const double* u0, const double* p, const double* tspan, const double* saveat, double* t_out,
                  double* u_out, int32_t* nsaved, int32_t* retcode, ode_stats* stats) {
    if (!h->copy_in) {
        CUDA_TRY(h, cudaStreamCreateWithFlags(&h->copy_in, cudaStreamNonBlocking));
        CUDA_TRY(h, cudaStreamCreateWithFlags(&h->copy_out, cudaStreamNonBlocking));
        for (int k = 0; k < kPipeChunks; ++k) {
            CUDA_TRY(h, cudaEventCreateWithFlags(&h->pipe_in[k], cudaEventDisableTiming));
            CUDA_TRY(h, cudaEventCreateWithFlags(&h->pipe_done[k], cudaEventDisableTiming));
        }
    }
    const size_t n = (size_t)d->n_states, np = (size_t)d->n_params, cap = save_cap(o), rows = out_rows(d, o);
    const size_t pitch = (size_t)N * 8;
    const bool per_traj = o->saveat_per_traj && o->nsave > 0;
    cudaStream_t s = h->main.stream, ci = h->copy_in, co = h->copy_out;
    double* du0 = (double*)h->b_u0.p;
    double* dp = (double*)h->b_p.p;
    double* dts = (double*)h->b_tspan.p;
    double* dsv = (double*)h->b_saveat.p;
    double* dt = (double*)h->b_t.p;
    double* du = (double*)h->b_u.p;
    int32_t* dns = (int32_t*)h->b_ns.p;
    int32_t* drc = (int32_t*)h->b_rc.p;
    ode_stats* dst = (ode_stats*)h->b_st.p;
    int32_t* dnpt = (int32_t*)h->b_npt.p;
    if (o->nsave > 0 && !per_traj)
        CUDA_TRY(h, cudaMemcpyAsync(dsv, saveat, (size_t)o->nsave * 8, cudaMemcpyHostToDevice, ci));
    const int64_t chunk = (N + kPipeChunks - 1) / kPipeChunks;
    int rc = ODE_OK;
    for (int k = 0; k < kPipeChunks && rc == ODE_OK; ++k) {
        const int64_t a0 = (int64_t)k * chunk;
        const int64_t cnt = std::min<int64_t>(chunk, N - a0);
        if (cnt <= 0) break;
        const size_t w = (size_t)cnt * 8;
        CUDA_TRY(h, cudaMemcpy2DAsync(du0 + a0, pitch, u0 + a0, pitch, w, n, cudaMemcpyHostToDevice, ci));
        CUDA_TRY(h, cudaMemcpy2DAsync(dp + a0, pitch, p + a0, pitch, w, np, cudaMemcpyHostToDevice, ci));
        CUDA_TRY(h, cudaMemcpy2DAsync(dts + a0, pitch, tspan + a0, pitch, w, 2, cudaMemcpyHostToDevice, ci));
        if (per_traj)
            CUDA_TRY(h, cudaMemcpy2DAsync(dsv + a0, pitch, saveat + a0, pitch, w, (size_t)o->nsave,
                                          cudaMemcpyHostToDevice, ci));
        if (npt) CUDA_TRY(h, cudaMemcpyAsync(dnpt + a0, npt + a0, (size_t)cnt * 4, cudaMemcpyHostToDevice, ci));
        CUDA_TRY(h, cudaEventRecord(h->pipe_in[k], ci));
        CUDA_TRY(h, cudaStreamWaitEvent(s, h->pipe_in[k], 0));
        if (k == 0) CUDA_TRY(h, cudaEventRecord(h->main.ev0, s));
        rc = run_ensemble(h, h->main, d, o, cnt, npt ? dnpt + a0 : nullptr, du0 + a0, dp + a0, dts + a0,
                          per_traj ? dsv + a0 : dsv, dt + a0, du + a0, dns + a0, drc + a0, (OdeStatsDev*)(dst + a0), s,
                          /*graph=*/false, /*stride=*/N, /*timing=*/false);
        if (rc) break;
        CUDA_TRY(h, cudaEventRecord(h->pipe_done[k], s));
        CUDA_TRY(h, cudaStreamWaitEvent(co, h->pipe_done[k], 0));
        if (t_out) CUDA_TRY(h, cudaMemcpy2DAsync(t_out + a0, pitch, dt + a0, pitch, w, cap, cudaMemcpyDeviceToHost, co));
        CUDA_TRY(h, cudaMemcpy2DAsync(u_out + a0, pitch, du + a0, pitch, w, cap * rows, cudaMemcpyDeviceToHost, co));
        CUDA_TRY(h, cudaMemcpyAsync(nsaved + a0, dns + a0, (size_t)cnt * 4, cudaMemcpyDeviceToHost, co));
        CUDA_TRY(h, cudaMemcpyAsync(retcode + a0, drc + a0, (size_t)cnt * 4, cudaMemcpyDeviceToHost, co));
        if (stats)
            CUDA_TRY(h, cudaMemcpyAsync(stats + a0, dst + a0, (size_t)cnt * sizeof(ode_stats), cudaMemcpyDeviceToHost, co));
    }
    if (rc == ODE_OK) CUDA_TRY(h, cudaEventRecord(h->main.ev1, s));
    cudaStreamSynchronize(s);
    cudaStreamSynchronize(ci);
    cudaError_t e = cudaStreamSynchronize(co);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(h, ODE_E_CUDA, std::string("pipeline: ") + cudaGetErrorString(e));
    float ms = 0;
    if (cudaEventElapsedTime(&ms, h->main.ev0, h->main.ev1) == cudaSuccess) h->last_ms = ms;
    return ODE_OK;
}

// Host-side check of per-trajectory sizes: each a size class and <= n_states.
int check_sizes(ode_handle* h, const ode_problem_desc* d, const int32_t* npt, int64_t N) {
    if (!npt) return ODE_OK;
    if (d->model_id != ODE_MODEL_DUFFING_CHAIN)
        return fail(h, ODE_E_UNSUPPORTED, "per-trajectory sizes are supported for DUFFING_CHAIN");
    for (int64_t j = 0; j < N; ++j) {
        const int n = npt[j];
        bool cls = false;
        for (int k = 0; k < kNumClasses; ++k) cls = cls || n == kClassStates[k];
        if (!cls || n > d->n_states) {
            char buf[160];
            std::snprintf(buf, sizeof buf, "n_per_traj[%lld] = %d: sizes must be 4, 8, 16, 32 or 64 and <= n_states",
                          (long long)j, n);
            return fail(h, ODE_E_INVALID, buf);
        }
    }
    return ODE_OK;
}

// Evaluation kernel for a dense solve: the model-free one for Tsit5 and
// Rodas5P, the model's Vern7 one at the FP64 integrator's lane layout.
const DenseVariant* find_dense(int alg, int model, int n) {
    int cnt = 0;
    const DenseVariant* all = dense_variants(&cnt);
    const DenseVariant* best = nullptr;
    for (int k = 0; k < cnt; ++k) {
        const DenseVariant& v = all[k];
        if (v.alg != alg) continue;
        if (v.model < 0) return &v;
        if (v.model != model || v.n != n) continue;
        if (!best || v.lanes == default_lanes(alg, n, ODE_PREC_FP64)) best = &v;
    }
    return best;
}

// Synchronous solve on host buffers (validated by the caller); k_out: dense
// output or nullptr.
int solve_host(ode_handle* h, const ode_problem_desc* d, const ode_options* o, int64_t N, const int32_t* npt,
               const double* u0, const double* p, const double* tspan, const double* saveat, double* t_out,
               double* u_out, double* k_out, int32_t* nsaved, int32_t* retcode, ode_stats* stats) {
    int rc = ODE_OK;
    std::lock_guard<std::mutex> lk(h->api_mu);
    CUDA_TRY(h, cudaSetDevice(h->device));
    *h->h_abort = 0;
    ode_options ostaged;
    if ((rc = stage_tstops(h, o, h->main.stream, &ostaged))) return rc;
    if ((rc = stage_tolvec(h, d, h->main.stream, &ostaged))) return rc;
    if (!ostaged.forward_only && N > 0) ostaged.forward_only = all_forward(tspan, N) ? 1 : 0;
    o = &ostaged;
    if (N > 0) {   // every buffer page-locked: the kernels work in place, no staging copies
        const double *mu0 = mapped_ptr(u0), *mp = mapped_ptr(p), *mts = mapped_ptr(tspan);
        const double* msv = o->nsave > 0 ? mapped_ptr(saveat) : nullptr;
        const int32_t* mnpt = npt ? mapped_ptr(npt) : nullptr;
        double *mt = t_out ? mapped_ptr(t_out) : nullptr, *mu = mapped_ptr(u_out);
        int32_t *mns = mapped_ptr(nsaved), *mrc = mapped_ptr(retcode);
        ode_stats* mst = stats ? mapped_ptr(stats) : nullptr;
        double* mk = k_out ? mapped_ptr(k_out) : nullptr;
        if (mu0 && mp && mts && mu && mns && mrc && (o->nsave == 0 || msv) && (!npt || mnpt) && (!t_out || mt) &&
            (!stats || mst) && (!k_out || mk)) {
            cudaStream_t s = h->main.stream;
            rc = run_ensemble(h, h->main, d, o, N, mnpt, mu0, mp, mts, msv, mt, mu, mns, mrc, (OdeStatsDev*)mst, s,
                              /*graph=*/true, 0, true, mk);
            cudaError_t e = cudaStreamSynchronize(s);
            if (rc) return rc;
            if (e != cudaSuccess) return fail(h, ODE_E_CUDA, std::string("solve: ") + cudaGetErrorString(e));
            float ms = 0;
            if (cudaEventElapsedTime(&ms, h->main.ev0, h->main.ev1) == cudaSuccess) h->last_ms = ms;
            return ODE_OK;
        }
    }
    const size_t n = (size_t)d->n_states, np = (size_t)d->n_params, cap = save_cap(o), rows = out_rows(d, o);
    const size_t nsv = (size_t)o->nsave * (o->saveat_per_traj ? (size_t)N : 1);
    if ((rc = grow(h, h->b_u0, n * N * 8)) || (rc = grow(h, h->b_p, np * N * 8)) ||
        (rc = grow(h, h->b_tspan, 2 * N * 8)) || (rc = grow(h, h->b_saveat, nsv * 8)) ||
        (rc = grow(h, h->b_t, cap * N * 8)) || (rc = grow(h, h->b_u, cap * rows * N * 8)) ||
        (rc = grow(h, h->b_ns, N * 4)) || (rc = grow(h, h->b_rc, N * 4)) ||
        (rc = grow(h, h->b_st, N * sizeof(ode_stats))) || (npt && (rc = grow(h, h->b_npt, N * 4))))
        return rc;
    const size_t kbytes = k_out ? cap * (size_t)kDenseVectors[d->alg_id] * n * N * 8 : 0;
    if (k_out && (rc = grow(h, h->b_k, kbytes))) return rc;
    cudaStream_t s = h->main.stream;
    if (!k_out && N >= kPipeMin && (cap * (n + 1) + n + np + 2) * 8 >= kPipeMinBytesPerTraj)
        return solve_chunked(h, d, o, N, npt, u0, p, tspan, saveat, t_out, u_out, nsaved, retcode, stats);
    CUDA_TRY(h, cudaMemcpyAsync(h->b_u0.p, u0, n * N * 8, cudaMemcpyHostToDevice, s));
    CUDA_TRY(h, cudaMemcpyAsync(h->b_p.p, p, np * N * 8, cudaMemcpyHostToDevice, s));
    CUDA_TRY(h, cudaMemcpyAsync(h->b_tspan.p, tspan, 2 * N * 8, cudaMemcpyHostToDevice, s));
    if (nsv) CUDA_TRY(h, cudaMemcpyAsync(h->b_saveat.p, saveat, nsv * 8, cudaMemcpyHostToDevice, s));
    if (npt) CUDA_TRY(h, cudaMemcpyAsync(h->b_npt.p, npt, N * 4, cudaMemcpyHostToDevice, s));
    rc = run_ensemble(h, h->main, d, o, N, npt ? (const int32_t*)h->b_npt.p : nullptr, (const double*)h->b_u0.p,
                      (const double*)h->b_p.p, (const double*)h->b_tspan.p, (const double*)h->b_saveat.p,
                      (double*)h->b_t.p, (double*)h->b_u.p, (int32_t*)h->b_ns.p, (int32_t*)h->b_rc.p,
                      (OdeStatsDev*)h->b_st.p, s, /*graph=*/true, 0, true, k_out ? (double*)h->b_k.p : nullptr);
    if (rc) {
        cudaStreamSynchronize(s);
        return rc;
    }
    if (t_out) CUDA_TRY(h, cudaMemcpyAsync(t_out, h->b_t.p, cap * N * 8, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(h, cudaMemcpyAsync(u_out, h->b_u.p, cap * rows * N * 8, cudaMemcpyDeviceToHost, s));
    if (k_out) CUDA_TRY(h, cudaMemcpyAsync(k_out, h->b_k.p, kbytes, cudaMemcpyDeviceToHost, s));
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
    std::vector<double> u0, p, tspan, saveat, tstops;   // tstops sorted; o.tstops is unused
    std::vector<int32_t> npt;
    std::vector<int32_t> save_idxs;                     // o.save_idxs is unused
    double* t_out = nullptr;
    double* u_out = nullptr;
    int32_t* nsaved = nullptr;
    int32_t* retcode = nullptr;
    ode_stats* stats = nullptr;
    int state = 0;  // 0 queued, 1 running, 2 done
    int status = ODE_OK;
    double t_submit = 0, t_start = 0, t_done = 0;   // CLOCK_MONOTONIC seconds
};

// One launch: a request, or several compatible ones merged into one ensemble
// (continuous batching inside the kernel: their trajectories share the launch,
// each with its own tolerances, and a lane group that finishes one request's
// trajectory goes on with another's).
struct Batch {
    std::vector<std::shared_ptr<Request>> reqs;
    std::vector<int64_t> offset;   // first trajectory of each request in the merged ensemble
    int64_t N = 0;
    int slot = -1;
    size_t bytes = 0;
    void* dmem = nullptr;          // one device block for the inputs and outputs
    int status = ODE_OK;
    const Request& head() const { return *reqs.front(); }
};

double mono_now() {
    timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Requests merge when they differ only in their trajectories and tolerances:
// same model, method, precision and sizes, the same options otherwise, the
// same shared saveat and tstops, and uniform sizes.
bool mergeable(const Request& a, const Request& b) {
    if (std::memcmp(&a.d, &b.d, sizeof(a.d)) != 0) return false;
    if (!a.npt.empty() || !b.npt.empty() || a.o.saveat_per_traj || b.o.saveat_per_traj) return false;
    ode_options x = a.o, y = b.o;
    x.reltol = y.reltol = 0.0;
    x.abstol = y.abstol = 0.0;
    if (std::memcmp(&x, &y, sizeof(x)) != 0) return false;
    return a.saveat == b.saveat && a.tstops == b.tstops && a.save_idxs == b.save_idxs;
}

// Byte offsets of one batch's block: inputs first, then outputs, so each
// direction is one contiguous copy.  The pinned staging of the slot and the
// device block share this layout.  Merged batches carry per-trajectory
// tolerances.
struct Layout {
    size_t u0, p, ts, rtol, atol, sv, tst, idx, npt, in_end, t, u, ns, rc, st, total;
};
Layout layout(const Request& h, int64_t Ntot, bool per_traj_tol) {
    const size_t n = (size_t)h.d.n_states, np = (size_t)h.d.n_params, N = (size_t)Ntot, cap = save_cap(&h.o);
    const size_t rows = out_rows(&h.d, &h.o);
    Layout L;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += align256(bytes); return o; };
    L.u0 = take(n * N * 8);
    L.p = take(np * N * 8);
    L.ts = take(2 * N * 8);
    L.rtol = per_traj_tol ? take(N * 8) : (size_t)-1;
    L.atol = per_traj_tol ? take(N * 8) : (size_t)-1;
    L.sv = take(std::max<size_t>(h.saveat.size(), 1) * 8);
    L.tst = take(std::max<size_t>(h.tstops.size(), 1) * 8);
    L.idx = take(std::max<size_t>(h.save_idxs.size(), 1) * 4);
    L.npt = h.npt.empty() ? (size_t)-1 : take(N * 4);
    L.in_end = off;
    L.t = take(cap * N * 8);
    L.u = take(cap * rows * N * 8);
    L.ns = take(N * 4);
    L.rc = take(N * 4);
    L.st = take(N * sizeof(ode_stats));
    L.total = off;
    return L;
}
Layout layout(const Batch& b) { return layout(b.head(), b.N, b.reqs.size() > 1); }

size_t request_bytes(const Request& r) { return layout(r, r.N, false).total; }

// Start batch b on slot k: stage every request's inputs at its offset in the
// slot's pinned buffer, one copy in, the ensemble kernel(s), one copy of the
// outputs back, all on the slot's stream.
int admit(ode_handle* h, Batch& b, int k) {
    Ctx& c = h->slot_ctx[k];
    cudaStream_t s = c.stream;
    const Request& r0 = b.head();
    const Layout L = layout(b);
    const size_t n = (size_t)r0.d.n_states, np = (size_t)r0.d.n_params, N = (size_t)b.N;
    if (h->slot_pinned_cap[k] < L.total) {
        if (h->slot_pinned[k]) cudaFreeHost(h->slot_pinned[k]);
        h->slot_pinned[k] = nullptr;
        h->slot_pinned_cap[k] = 0;
        const size_t want = std::max<size_t>(L.total, (size_t)1 << 20);
        CUDA_TRY(h, cudaHostAlloc(&h->slot_pinned[k], want, cudaHostAllocDefault));
        h->slot_pinned_cap[k] = want;
    }
    char* hs = (char*)h->slot_pinned[k];
    // structure-of-arrays rows: request q's trajectories at columns [offset, offset + N_q)
    auto pack = [&](size_t base, size_t rows, const std::vector<double>& src, const Request& r, int64_t off) {
        for (size_t i = 0; i < rows; ++i)
            std::memcpy(hs + base + (i * N + (size_t)off) * 8, src.data() + i * (size_t)r.N, (size_t)r.N * 8);
    };
    for (size_t q = 0; q < b.reqs.size(); ++q) {
        const Request& r = *b.reqs[q];
        const int64_t off = b.offset[q];
        pack(L.u0, n, r.u0, r, off);
        pack(L.p, np, r.p, r, off);
        pack(L.ts, 2, r.tspan, r, off);
        if (b.reqs.size() > 1) {
            std::fill((double*)(hs + L.rtol) + off, (double*)(hs + L.rtol) + off + r.N, r.o.reltol);
            std::fill((double*)(hs + L.atol) + off, (double*)(hs + L.atol) + off + r.N, r.o.abstol);
        }
    }
    if (!r0.saveat.empty()) std::memcpy(hs + L.sv, r0.saveat.data(), r0.saveat.size() * 8);
    if (!r0.tstops.empty()) std::memcpy(hs + L.tst, r0.tstops.data(), r0.tstops.size() * 8);
    if (!r0.save_idxs.empty()) std::memcpy(hs + L.idx, r0.save_idxs.data(), r0.save_idxs.size() * 4);
    if (!r0.npt.empty()) std::memcpy(hs + L.npt, r0.npt.data(), N * 4);
    CUDA_TRY(h, cudaMallocAsync(&b.dmem, L.total, s));
    char* base = (char*)b.dmem;
    CUDA_TRY(h, cudaMemcpyAsync(base, hs, L.in_end, cudaMemcpyHostToDevice, s));
    ode_options o = r0.o;
    o.ntstops = (int32_t)r0.tstops.size();
    o.tstops = r0.tstops.empty() ? nullptr : (const double*)(base + L.tst);
    o.save_idxs = r0.save_idxs.empty() ? nullptr : (const int32_t*)(base + L.idx);
    const bool pt = b.reqs.size() > 1;
    int rc = run_ensemble(h, c, &r0.d, &o, b.N, r0.npt.empty() ? nullptr : (const int32_t*)(base + L.npt),
                          (const double*)(base + L.u0), (const double*)(base + L.p), (const double*)(base + L.ts),
                          (const double*)(base + L.sv), (double*)(base + L.t), (double*)(base + L.u),
                          (int32_t*)(base + L.ns), (int32_t*)(base + L.rc), (OdeStatsDev*)(base + L.st), s,
                          /*graph=*/false, 0, /*timing=*/false, nullptr,
                          pt ? (const double*)(base + L.rtol) : nullptr, pt ? (const double*)(base + L.atol) : nullptr);
    if (rc) return rc;
    CUDA_TRY(h, cudaMemcpyAsync(hs + L.t, base + L.t, L.total - L.t, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(h, cudaFreeAsync(b.dmem, s));
    b.dmem = nullptr;
    CUDA_TRY(h, cudaEventRecord(h->slot_ev[k], s));
    return ODE_OK;
}

// Outputs from the slot's staging into each request's buffers.
void finish(ode_handle* h, Batch& b) {
    const Request& r0 = b.head();
    const size_t rows = out_rows(&r0.d, &r0.o), N = (size_t)b.N, cap = save_cap(&r0.o);
    if (b.status == ODE_OK && b.slot >= 0 && h->slot_pinned[b.slot]) {
        const Layout L = layout(b);
        const char* hs = (const char*)h->slot_pinned[b.slot];
        for (size_t q = 0; q < b.reqs.size(); ++q) {
            Request& r = *b.reqs[q];
            const size_t off = (size_t)b.offset[q], m = (size_t)r.N;
            if (r.t_out)
                for (size_t i = 0; i < cap; ++i) std::memcpy(r.t_out + i * m, hs + L.t + (i * N + off) * 8, m * 8);
            for (size_t i = 0; i < cap * rows; ++i) std::memcpy(r.u_out + i * m, hs + L.u + (i * N + off) * 8, m * 8);
            std::memcpy(r.nsaved, hs + L.ns + off * 4, m * 4);
            std::memcpy(r.retcode, hs + L.rc + off * 4, m * 4);
            if (r.stats) std::memcpy(r.stats, hs + L.st + off * sizeof(ode_stats), m * sizeof(ode_stats));
        }
    }
    for (auto& rp : b.reqs) {
        Request& r = *rp;
        if (r.status == ODE_OK) r.status = b.status;
        r.u0.clear(); r.u0.shrink_to_fit();
        r.p.clear(); r.p.shrink_to_fit();
        r.tspan.clear(); r.tspan.shrink_to_fit();
    }
}

// Book-keeping of a finished request (lock held).
void retire(ode_handle* h, const std::shared_ptr<Request>& r) {
    r->state = 2;
    r->t_done = mono_now();
    h->n_completed++;
    h->completed.push_back(r->ticket);
}
void retire(ode_handle* h, Batch& b) {
    if (b.slot >= 0) h->slot_busy[b.slot] = 0;
    h->hbm_in_use -= b.bytes;
    for (auto& r : b.reqs) retire(h, r);
}

// A request that has waited this long at the head of the queue holds back
// the admission of the requests behind it until it fits (no starvation).
constexpr double kServeAgingSeconds = 0.25;
// At most this many trajectories are merged into one launch.
constexpr int64_t kServeMaxBatchTraj = 1 << 17;

// The serving loop: retire finished batches, then admit queued requests while
// a slot is free and the HBM budget allows.  A request is merged with every
// queued request it is compatible with (up to kServeMaxBatchTraj
// trajectories); a request that does not fit does not block the smaller ones
// behind it, unless it has waited kServeAgingSeconds.  A request larger than
// the whole budget is rejected with ODE_E_NOMEM.  Copies into and out of the
// pinned staging run without the lock, so submitters are not held up.
void serve_loop(ode_handle* h) {
    cudaSetDevice(h->device);
    std::unique_lock<std::mutex> lk(h->mu);
    std::vector<std::shared_ptr<Batch>> done;
    std::vector<std::shared_ptr<Batch>> starts;
    while (!h->stop) {
        bool progressed = false;
        done.clear();
        for (size_t i = 0; i < h->running.size();) {
            auto b = h->running[i];
            cudaError_t q = cudaEventQuery(h->slot_ev[b->slot]);
            if (q == cudaErrorNotReady) { ++i; continue; }
            if (q != cudaSuccess) b->status = ODE_E_CUDA;
            done.push_back(b);
            h->running.erase(h->running.begin() + i);
        }
        if (!done.empty()) {
            lk.unlock();
            for (auto& b : done) finish(h, *b);
            lk.lock();
            for (auto& b : done) retire(h, *b);
            progressed = true;
        }
        starts.clear();
        const double now = mono_now();
        for (auto it = h->pending.begin(); it != h->pending.end();) {
            auto r = *it;
            if (r->state != 0) { it = h->pending.erase(it); continue; }   // merged into an earlier batch
            const size_t rb = request_bytes(*r);
            if (rb > h->budget) {
                it = h->pending.erase(it);
                r->status = ODE_E_NOMEM;
                h->n_rejected++;
                retire(h, r);
                progressed = true;
                continue;
            }
            int k = -1;
            for (int sl = 0; sl < (int)h->slot_ctx.size(); ++sl)
                if (!h->slot_busy[sl]) { k = sl; break; }
            if (k < 0) break;
            if (h->hbm_in_use + rb > h->budget) {
                if (now - r->t_submit > kServeAgingSeconds) break;   // it waits no longer behind others
                ++it;
                continue;
            }
            auto b = std::make_shared<Batch>();
            b->reqs.push_back(r);
            b->offset.push_back(0);
            b->N = r->N;
            b->bytes = rb;
            r->state = 1;
            it = h->pending.erase(it);
            // merge compatible requests queued behind it while the budget allows
            for (auto jt = it; jt != h->pending.end() && b->N < kServeMaxBatchTraj; ++jt) {
                auto& q = *jt;
                if (q->state != 0 || !mergeable(*r, *q) || b->N + q->N > kServeMaxBatchTraj) continue;
                const size_t nb = layout(*r, b->N + q->N, true).total;
                if (h->hbm_in_use + nb > h->budget) continue;
                b->offset.push_back(b->N);
                b->reqs.push_back(q);
                b->N += q->N;
                b->bytes = nb;
                q->state = 1;
            }
            b->slot = k;
            h->slot_busy[k] = 1;
            h->hbm_in_use += b->bytes;
            h->n_admitted += (long long)b->reqs.size();
            h->n_batches++;
            starts.push_back(b);
        }
        if (!starts.empty()) {
            lk.unlock();
            for (auto& b : starts) {
                const double t = mono_now();
                for (auto& r : b->reqs) r->t_start = t;
                int rc = admit(h, *b, b->slot);
                if (rc) {
                    b->status = rc;
                    cudaStreamSynchronize(h->slot_ctx[b->slot].stream);
                    if (b->dmem) cudaFree(b->dmem);
                    b->dmem = nullptr;
                }
            }
            lk.lock();
            for (auto& b : starts) {
                if (b->status != ODE_OK) {
                    for (auto& r : b->reqs) r->status = b->status;
                    retire(h, *b);
                } else {
                    h->running.push_back(b);
                }
            }
            progressed = true;
        }
        if (progressed) h->cv.notify_all();
        if (h->running.empty() && h->pending.empty())
            h->cv.wait(lk, [&] { return h->stop || !h->pending.empty(); });
        else if (!progressed)
            h->cv.wait_for(lk, std::chrono::microseconds(20));
    }
}

int ensure_worker(ode_handle* h) {
    if (h->worker_started) return ODE_OK;
    h->slot_ctx.resize(h->slots);
    h->slot_busy.assign(h->slots, 0);
    h->slot_pinned.assign(h->slots, nullptr);
    h->slot_pinned_cap.assign(h->slots, 0);
    h->slot_ev.assign(h->slots, nullptr);
    for (int k = 0; k < h->slots; ++k) {
        int rc = ctx_init(h, h->slot_ctx[k], nullptr);
        if (rc) return rc;
        CUDA_TRY(h, cudaEventCreateWithFlags(&h->slot_ev[k], cudaEventDisableTiming));
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
    o->interp_points = 10;
    o->max_jac_age = 1;
    o->jac_reuse_gamma_tol = 0.03;
    o->adaptive = 1;
    o->controller_given = 0;
    o->beta1 = o->beta2 = o->qoldinit = o->qmin = o->gamma = o->qsteady_min = o->qsteady_max = std::nan("");
}

size_t ode_options_size(void) { return sizeof(ode_options); }
size_t ode_problem_desc_size(void) { return sizeof(ode_problem_desc); }

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
    for (auto& r : h->running) finish(h, *r);
    for (DevBuf* b : {&h->b_u0, &h->b_p, &h->b_tspan, &h->b_saveat, &h->b_tstops, &h->b_idx, &h->b_atol, &h->b_rtol, &h->b_t, &h->b_u, &h->b_ns, &h->b_rc,
                      &h->b_st, &h->b_npt})
        if (b->p) cudaFree(b->p);
    ctx_free(h->main);
    for (auto& c : h->slot_ctx) ctx_free(c);
    for (void* q : h->slot_pinned)
        if (q) cudaFreeHost(q);
    for (int k = 0; k < 4; ++k) {
        if (h->pipe_in[k]) cudaEventDestroy(h->pipe_in[k]);
        if (h->pipe_done[k]) cudaEventDestroy(h->pipe_done[k]);
    }
    if (h->copy_in) cudaStreamDestroy(h->copy_in);
    if (h->copy_out) cudaStreamDestroy(h->copy_out);
    for (cudaEvent_t e : h->slot_ev)
        if (e) cudaEventDestroy(e);
    if (h->h_abort) cudaFreeHost(h->h_abort);
    delete h;
}

int ode_solve_ensemble_device(ode_handle* h, const ode_problem_desc* d, const ode_options* o, int64_t N,
                              const int32_t* npt_dev, const double* u0, const double* p, const double* tspan,
                              const double* saveat, double* t_out, double* u_out, int32_t* nsaved,
                              int32_t* retcode, ode_stats* stats, void* cuda_stream) {
    int rc = validate(h, d, o, N);
    if (rc) return rc;
    if (N > 0 && (!u0 || !p || !tspan || !u_out || !nsaved || !retcode))
        return fail(h, ODE_E_INVALID, "null input or output buffer");
    if (o->nsave > 0 && !saveat) return fail(h, ODE_E_INVALID, "nsave > 0 but saveat is null");
    std::lock_guard<std::mutex> lk(h->api_mu);
    CUDA_TRY(h, cudaSetDevice(h->device));
    *h->h_abort = 0;
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : h->main.stream;
    return run_ensemble(h, h->main, d, o, N, npt_dev, u0, p, tspan, saveat, t_out, u_out, nsaved, retcode,
                        (OdeStatsDev*)stats, s, /*graph=*/true);
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
    if ((rc = check_sizes(h, d, npt, N))) return rc;
    if ((rc = check_host_tstops(h, o)) || (rc = check_host_save_idxs(h, d, o)) || (rc = check_host_tolvec(h, d, o)))
        return rc;
    return solve_host(h, d, o, N, npt, u0, p, tspan, saveat, t_out, u_out, nullptr, nsaved, retcode, stats);
}

int ode_dense_nk(int alg) {
    return alg >= ODE_TSIT5 && alg < kNumAlgs ? kDenseVectors[alg] : ODE_E_INVALID;
}

int ode_solve_ensemble_dense(ode_handle* h, const ode_problem_desc* d, const ode_options* o, int64_t N,
                             const double* u0, const double* p, const double* tspan, double* t_out,
                             double* u_out, double* k_out, int32_t* nsaved, int32_t* retcode, ode_stats* stats) {
    int rc = validate(h, d, o, N);
    if (rc) return rc;
    if (!o->save_everystep || o->nsave != 0)
        return fail(h, ODE_E_INVALID, "dense output saves every step: save_everystep = 1 and nsave = 0");
    if (kDenseVectors[d->alg_id] == 0) return fail(h, ODE_E_UNSUPPORTED, "no dense output for this method");
    if (o->nsave_idxs > 0) return fail(h, ODE_E_UNSUPPORTED, "save_idxs with dense output is not supported");
    if (N > 0 && (!u0 || !p || !tspan || !u_out || !k_out || !nsaved || !retcode))
        return fail(h, ODE_E_INVALID, "null input or output buffer");
    if ((rc = check_host_tstops(h, o))) return rc;
    return solve_host(h, d, o, N, nullptr, u0, p, tspan, nullptr, t_out, u_out, k_out, nsaved, retcode, stats);
}

int ode_dense_eval_deriv(ode_handle* h, const ode_problem_desc* d, int64_t N, const double* p,
                         const double* t_saved, const double* u_saved, const double* k_saved, const int32_t* nsaved,
                         int32_t cap, int32_t nq, const double* tq, int32_t tq_per_traj, int32_t deriv, double* out) {
    return ode_dense_eval_ex(h, d, N, p, t_saved, u_saved, k_saved, nsaved, cap, nq, tq, tq_per_traj, deriv, 0, out);
}

int ode_dense_eval_ex(ode_handle* h, const ode_problem_desc* d, int64_t N, const double* p,
                      const double* t_saved, const double* u_saved, const double* k_saved, const int32_t* nsaved,
                      int32_t cap, int32_t nq, const double* tq, int32_t tq_per_traj, int32_t deriv,
                      int32_t continuity_right, double* out) {
    if (!h || !d) return fail(h, ODE_E_INVALID, "null handle or problem");
    if (deriv < 0) return fail(h, ODE_E_INVALID, "negative derivative order");
    if (deriv > 3) return fail(h, ODE_E_UNSUPPORTED, "dense evaluation of the value (0) or derivatives 1 to 3 only");
    // the reference's interpolants have Val{2} and Val{3} forms for Tsit5 and the
    // Rosenbrock combined tableaus (Rodas5P), not for Vern7 or Rosenbrock23
    if (deriv >= 2 && d->alg_id != ODE_TSIT5 && d->alg_id != ODE_RODAS5P)
        return fail(h, ODE_E_UNSUPPORTED, "derivatives 2 and 3 are for Tsit5 and Rodas5P solutions");
    ode_options o;
    ode_options_default(&o);
    int rc = validate(h, d, &o, N);
    if (rc) return rc;
    if (cap < 1 || nq < 0) return fail(h, ODE_E_INVALID, "cap must be >= 1 and nq >= 0");
    if (N == 0 || nq == 0) return ODE_OK;
    if (!p || !t_saved || !u_saved || !k_saved || !nsaved || !tq || !out)
        return fail(h, ODE_E_INVALID, "null input or output buffer");
    for (int64_t j = 0; j < N; ++j)
        if (nsaved[j] < 0 || nsaved[j] > cap) return fail(h, ODE_E_INVALID, "nsaved outside [0, cap]");
    const DenseVariant* v = find_dense(d->alg_id, d->model_id, d->n_states);
    if (!v) {
        char buf[128];
        std::snprintf(buf, sizeof buf, "no dense evaluation kernel for alg %d model %d n %d", d->alg_id,
                      d->model_id, d->n_states);
        return fail(h, ODE_E_UNSUPPORTED, buf);
    }
    const size_t n = (size_t)d->n_states, np = (size_t)d->n_params, nk = (size_t)kDenseVectors[d->alg_id];
    const size_t ntq = (size_t)nq * (tq_per_traj ? (size_t)N : 1);
    std::lock_guard<std::mutex> lk(h->api_mu);
    CUDA_TRY(h, cudaSetDevice(h->device));
    DenseArgs a;
    a.N = N;
    a.n = d->n_states;
    a.nq = nq;
    a.tq_per_traj = tq_per_traj ? 1 : 0;
    a.cap = cap;
    a.deriv = deriv;
    a.right = continuity_right ? 1 : 0;
    cudaStream_t s = h->main.stream;
    // The saves are copied in (the interval search reads them scattered, which is
    // slow from host memory: measured 30x slower in place over NVLink-C2C); a
    // page-locked `out` is written in place, coalesced.
    double* mout = mapped_ptr(out);
    const bool in_place = mout != nullptr;
    if ((rc = grow(h, h->b_p, np * N * 8)) || (rc = grow(h, h->b_t, (size_t)cap * N * 8)) ||
        (rc = grow(h, h->b_u, (size_t)cap * n * N * 8)) || (rc = grow(h, h->b_k, (size_t)cap * nk * n * N * 8)) ||
        (rc = grow(h, h->b_ns, N * 4)) || (rc = grow(h, h->b_tq, ntq * 8)) ||
        (!in_place && (rc = grow(h, h->b_out, (size_t)nq * n * N * 8))))
        return rc;
    CUDA_TRY(h, cudaMemcpyAsync(h->b_p.p, p, np * N * 8, cudaMemcpyHostToDevice, s));
    CUDA_TRY(h, cudaMemcpyAsync(h->b_t.p, t_saved, (size_t)cap * N * 8, cudaMemcpyHostToDevice, s));
    CUDA_TRY(h, cudaMemcpyAsync(h->b_u.p, u_saved, (size_t)cap * n * N * 8, cudaMemcpyHostToDevice, s));
    CUDA_TRY(h, cudaMemcpyAsync(h->b_k.p, k_saved, (size_t)cap * nk * n * N * 8, cudaMemcpyHostToDevice, s));
    CUDA_TRY(h, cudaMemcpyAsync(h->b_ns.p, nsaved, N * 4, cudaMemcpyHostToDevice, s));
    CUDA_TRY(h, cudaMemcpyAsync(h->b_tq.p, tq, ntq * 8, cudaMemcpyHostToDevice, s));
    a.p = (const double*)h->b_p.p;
    a.ts = (const double*)h->b_t.p;
    a.us = (const double*)h->b_u.p;
    a.ks = (const double*)h->b_k.p;
    a.nsaved = (const int32_t*)h->b_ns.p;
    a.tq = (const double*)h->b_tq.p;
    a.out = in_place ? mout : (double*)h->b_out.p;
    const int block = 128;
    const long long threads = (long long)N * nq * v->lanes;
    const long long grid = (threads + block - 1) / block;
    if (grid > 0x7fffffffLL) return fail(h, ODE_E_INVALID, "too many (trajectory, query) pairs for one launch");
    CUDA_TRY(h, cudaEventRecord(h->main.ev0, s));
    v->launch(a, (int)grid, block, s);
    CUDA_TRY(h, cudaGetLastError());
    h->launches++;
    CUDA_TRY(h, cudaEventRecord(h->main.ev1, s));
    if (!in_place) CUDA_TRY(h, cudaMemcpyAsync(out, h->b_out.p, (size_t)nq * n * N * 8, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(h, cudaStreamSynchronize(s));
    float ms = 0;
    if (cudaEventElapsedTime(&ms, h->main.ev0, h->main.ev1) == cudaSuccess) h->last_ms = ms;
    return ODE_OK;
}

int ode_dense_eval(ode_handle* h, const ode_problem_desc* d, int64_t N, const double* p, const double* t_saved,
                   const double* u_saved, const double* k_saved, const int32_t* nsaved, int32_t cap, int32_t nq,
                   const double* tq, int32_t tq_per_traj, double* out) {
    return ode_dense_eval_deriv(h, d, N, p, t_saved, u_saved, k_saved, nsaved, cap, nq, tq, tq_per_traj, 0, out);
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
    if ((rc = check_sizes(h, d, npt, N))) return rc;
    if (o->abstol_vec || o->reltol_vec)
        return fail(h, ODE_E_UNSUPPORTED, "per-state tolerances are not taken by the serving queue");
    if ((rc = check_host_tstops(h, o)) || (rc = check_host_save_idxs(h, d, o))) return rc;
    auto r = std::make_shared<Request>();
    r->d = *d;
    r->o = *o;
    r->tstops = sorted_tstops(o);
    r->o.tstops = nullptr;
    r->o.ntstops = (int32_t)r->tstops.size();
    if (o->nsave_idxs > 0) r->save_idxs.assign(o->save_idxs, o->save_idxs + o->nsave_idxs);
    r->o.save_idxs = nullptr;
    r->N = N;
    const size_t n = (size_t)d->n_states, np = (size_t)d->n_params;
    r->u0.assign(u0, u0 + n * N);
    r->p.assign(p, p + np * N);
    r->tspan.assign(tspan, tspan + 2 * N);
    if (!r->o.forward_only && N > 0) r->o.forward_only = all_forward(tspan, N) ? 1 : 0;
    if (o->nsave > 0) r->saveat.assign(saveat, saveat + (size_t)o->nsave * (o->saveat_per_traj ? (size_t)N : 1));
    if (npt) r->npt.assign(npt, npt + N);
    r->t_out = t_out;
    r->u_out = u_out;
    r->nsaved = nsaved;
    r->retcode = retcode;
    r->stats = stats;
    std::unique_lock<std::mutex> lk(h->mu);
    if (h->max_queued > 0 && h->pending.size() >= h->max_queued)
        return fail(h, ODE_E_BUSY, "serving queue full (ode_set_serving_queue_limit)");
    CUDA_TRY(h, cudaSetDevice(h->device));
    rc = ensure_worker(h);
    if (rc) return rc;
    r->ticket = h->next_ticket++;
    r->t_submit = mono_now();
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

int ode_next_completed(ode_handle* h, double timeout_s, uint64_t* ticket, int32_t* status, double* times) {
    if (!h || !ticket) return fail(h, ODE_E_INVALID, "null handle or ticket pointer");
    std::unique_lock<std::mutex> lk(h->mu);
    *ticket = 0;
    auto ready = [&] {
        while (!h->completed.empty() && !h->tickets.count(h->completed.front())) h->completed.pop_front();
        return !h->completed.empty();
    };
    if (timeout_s < 0) h->cv.wait(lk, ready);
    else if (timeout_s > 0) h->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), ready);
    if (!ready()) return ODE_OK;
    const uint64_t t = h->completed.front();
    h->completed.pop_front();
    auto r = h->tickets[t];
    h->tickets.erase(t);
    *ticket = t;
    if (status) *status = r->status;
    if (times) {
        times[0] = r->t_submit;
        times[1] = r->t_start;
        times[2] = r->t_done;
    }
    return ODE_OK;
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
    s->launches = (int32_t)std::min<long long>(h->n_batches, 0x7fffffff);
    return ODE_OK;
}

int ode_set_serving_queue_limit(ode_handle* h, int64_t max_queued) {
    if (!h || max_queued < 0) return fail(h, ODE_E_INVALID, "null handle or negative limit");
    std::unique_lock<std::mutex> lk(h->mu);
    h->max_queued = (size_t)max_queued;
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

int ode_autotune(ode_handle* h, const ode_problem_desc* d, const ode_options* o, int64_t N, const double* u0,
                 const double* p, const double* tspan, const double* saveat, int32_t* lanes_out,
                 int32_t* block_out, int32_t* scheduler_out, double* ms_out) {
    int rc = validate(h, d, o, N);
    if (rc) return rc;
    if (N <= 0 || !u0 || !p || !tspan) return fail(h, ODE_E_INVALID, "autotune needs a non-empty sample");
    if (o->nsave > 0 && !saveat) return fail(h, ODE_E_INVALID, "nsave > 0 but saveat is null");
    if ((rc = check_host_tstops(h, o)) || (rc = check_host_save_idxs(h, d, o)) || (rc = check_host_tolvec(h, d, o)))
        return rc;
    std::lock_guard<std::mutex> lk(h->api_mu);
    CUDA_TRY(h, cudaSetDevice(h->device));
    *h->h_abort = 0;
    ode_options ostaged;
    if ((rc = stage_tstops(h, o, h->main.stream, &ostaged))) return rc;
    if ((rc = stage_tolvec(h, d, h->main.stream, &ostaged))) return rc;
    if (!ostaged.forward_only) ostaged.forward_only = all_forward(tspan, N) ? 1 : 0;
    o = &ostaged;
    const size_t n = (size_t)d->n_states, np = (size_t)d->n_params, cap = save_cap(o), rows = out_rows(d, o);
    const size_t nsv = (size_t)o->nsave * (o->saveat_per_traj ? (size_t)N : 1);
    if ((rc = grow(h, h->b_u0, n * N * 8)) || (rc = grow(h, h->b_p, np * N * 8)) ||
        (rc = grow(h, h->b_tspan, 2 * N * 8)) || (rc = grow(h, h->b_saveat, nsv * 8)) ||
        (rc = grow(h, h->b_t, cap * N * 8)) || (rc = grow(h, h->b_u, cap * rows * N * 8)) ||
        (rc = grow(h, h->b_ns, N * 4)) || (rc = grow(h, h->b_rc, N * 4)) ||
        (rc = grow(h, h->b_st, N * sizeof(ode_stats))))
        return rc;
    cudaStream_t s = h->main.stream;
    CUDA_TRY(h, cudaMemcpyAsync(h->b_u0.p, u0, n * N * 8, cudaMemcpyHostToDevice, s));
    CUDA_TRY(h, cudaMemcpyAsync(h->b_p.p, p, np * N * 8, cudaMemcpyHostToDevice, s));
    CUDA_TRY(h, cudaMemcpyAsync(h->b_tspan.p, tspan, 2 * N * 8, cudaMemcpyHostToDevice, s));
    if (nsv) CUDA_TRY(h, cudaMemcpyAsync(h->b_saveat.p, saveat, nsv * 8, cudaMemcpyHostToDevice, s));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CUDA_TRY(h, cudaEventCreate(&e0));
    CUDA_TRY(h, cudaEventCreate(&e1));
    Ctx& c = h->main;
    double best = -1.0;
    ode_handle::Tuned pick{0, 0, 0, 0.0};
    const int blocks[3] = {32, 64, 128};
    rc = ODE_OK;
    for (const auto& v : all_variants()) {
        if (v.alg != d->alg_id || v.model != d->model_id || v.prec != d->precision || v.n != d->n_states) continue;
        for (int bi = 0; bi < 3 && rc == ODE_OK; ++bi) {
            for (int sched = 1; sched <= 2 && rc == ODE_OK; ++sched) {
                ode_options ot = *o;
                ot.lanes_per_traj = v.lanes;
                ot.block_size = blocks[bi];
                ot.scheduler = sched;
                double ms = 0.0;
                for (int rep = 0; rep < 3 && rc == ODE_OK; ++rep) {   // one warm-up, two timed
                    if (cudaEventRecord(e0, s) != cudaSuccess) { rc = fail(h, ODE_E_CUDA, "event record"); break; }
                    rc = run_ensemble(h, c, d, &ot, N, nullptr, (const double*)h->b_u0.p, (const double*)h->b_p.p,
                                      (const double*)h->b_tspan.p, (const double*)h->b_saveat.p, (double*)h->b_t.p,
                                      (double*)h->b_u.p, (int32_t*)h->b_ns.p, (int32_t*)h->b_rc.p,
                                      (OdeStatsDev*)h->b_st.p, s);
                    if (rc) break;
                    float f = 0.0f;
                    if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                        cudaEventElapsedTime(&f, e0, e1) != cudaSuccess) {
                        rc = fail(h, ODE_E_CUDA, "autotune timing");
                        break;
                    }
                    if (rep > 0) ms += 0.5 * f;
                }
                if (rc == ODE_OK && (best < 0.0 || ms < best)) {
                    best = ms;
                    pick = {v.lanes, blocks[bi], sched, ms};
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (best < 0.0) return fail(h, ODE_E_UNSUPPORTED, "no compiled kernel for this problem");
    {
        std::lock_guard<std::mutex> tl(h->tune_mu);
        h->tuned[std::make_tuple(d->alg_id, d->model_id, d->precision, d->n_states)] = pick;
    }
    if (lanes_out) *lanes_out = pick.lanes;
    if (block_out) *block_out = pick.block;
    if (scheduler_out) *scheduler_out = pick.scheduler;
    if (ms_out) *ms_out = pick.ms;
    return ODE_OK;
}

int ode_register_model(const char* source, const char* name, int32_t n_states, int32_t n_params, int32_t flags,
                       int32_t* model_id) {
    if (!model_id) return fail(nullptr, ODE_E_INVALID, "null model_id pointer");
    std::string why;
    int id = 0;
    const int rc = rtc_register(source, name, n_states, n_params, flags, &id, &why);
    if (rc) return fail(nullptr, rc, why);
    *model_id = id;
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
// [0, kCounters) the counters of a context (layout of kOff*), then
// [kCounters, kCounters + kNoAllocMaxTraj) bucketed trajectory indices.
// 8 MiB + 512 B, held by every GPU that loads the library until the process exits.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kCounters + kNoAllocMaxTraj];

std::mutex g_noalloc_mu;
struct NoallocCache {
    unsigned long long ctx_id = 0;   // the context the address was resolved in (0: none yet)
    unsigned long long* ptr = nullptr;
};
NoallocCache g_noalloc_cache[64];

// Identity of the current context (cuCtxGetCurrent + cuCtxGetId, reached through
// the runtime's driver entry points so the library needs no link to libcuda).
// A device reset in the caller's process destroys the primary context; the next
// one gets a new id, so the cached address is resolved again there.
int current_context_id(unsigned long long* id) {
    typedef int (*GetCurrent)(void**);
    typedef int (*GetId)(void*, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    if (!get_current || !get_id) {
        void* f0 = nullptr;
        void* f1 = nullptr;
        cudaDriverEntryPointQueryResult q0, q1;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0);
        if (e == cudaSuccess)
            e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1);
        if (e != cudaSuccess || !f0 || !f1 || q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess)
            return fail(nullptr, ODE_E_CUDA, "driver entry points cuCtxGetCurrent/cuCtxGetId not found");
        get_current = (GetCurrent)f0;
        get_id = (GetId)f1;
    }
    void* ctx = nullptr;
    if (get_current(&ctx) != 0 || ctx == nullptr || get_id(ctx, id) != 0)
        return fail(nullptr, ODE_E_CUDA, "no current CUDA context");
    return ODE_OK;
}

// Device address of the scratch for the current device, resolved with that
// device current and cached per device; resolved again when the device's
// context changed since (after a cudaDeviceReset).  cudaSetDevice on the
// current device makes its primary context current (initialising it if needed)
// and allocates nothing.
int noalloc_scratch(int dev, unsigned long long** out) {
    if (dev < 0 || dev >= 64) return fail(nullptr, ODE_E_INVALID, "device ordinal out of range");
    cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) return fail(nullptr, ODE_E_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    unsigned long long id = 0;
    int rc = current_context_id(&id);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoallocCache& c = g_noalloc_cache[dev];
    if (!c.ptr || c.ctx_id != id) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || ptr == nullptr)
            return fail(nullptr, ODE_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        c.ptr = (unsigned long long*)ptr;
        c.ctx_id = id;
    }
    *out = c.ptr;
    return ODE_OK;
}

int noalloc_launch(const KernelVariant* v, EnsembleArgs a, unsigned long long* queue, int sm_count, cudaStream_t s) {
    if (a.count <= 0) return ODE_OK;
    int block = 0;
    size_t smem = 0;
    cudaError_t e = launch_geometry(v, 0, &block, &smem);
    if (e != cudaSuccess) return fail(nullptr, ODE_E_CUDA, std::string("shared memory: ") + cudaGetErrorString(e));
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel_fn(v, a), block, smem);
    if (e != cudaSuccess) return fail(nullptr, ODE_E_CUDA, std::string("occupancy: ") + cudaGetErrorString(e));
    if (per_sm <= 0) per_sm = 1;
    long long want = (a.count * v->lanes + block - 1) / block;
    int grid = (int)std::min<long long>((long long)per_sm * sm_count, want);
    if (grid < 1) grid = 1;
    a.persistent = 1;
    a.refill_lanes = 16;
    a.queue = queue;
    launch_any(v, a, grid, block, smem, s);
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
    const char* why = "";
    int rc = check_problem(d, o, N, &why);
    if (rc) return fail(nullptr, rc, why);
    if (npt_dev && N > kNoAllocMaxTraj) {
        char buf[160];
        std::snprintf(buf, sizeof buf,
                      "ode_solve_ensemble_noalloc: %lld trajectories with per-trajectory sizes exceed the "
                      "fixed scratch maximum of %lld",
                      (long long)N, (long long)kNoAllocMaxTraj);
        return fail(nullptr, ODE_E_INVALID, buf);
    }
    if (npt_dev && d->model_id != ODE_MODEL_DUFFING_CHAIN)
        return fail(nullptr, ODE_E_UNSUPPORTED, "per-trajectory sizes are supported for DUFFING_CHAIN");
    if (N > 0 && (!u0 || !p || !tspan || !u_out || !nsaved || !retcode))
        return fail(nullptr, ODE_E_INVALID, "null input or output buffer");
    if (o->nsave > 0 && !saveat) return fail(nullptr, ODE_E_INVALID, "nsave > 0 but saveat is null");
    if (N == 0) return ODE_OK;
    int dev = 0, sm_count = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return fail(nullptr, ODE_E_CUDA, std::string("device query: ") + cudaGetErrorString(e));
    unsigned long long* scratch = nullptr;
    rc = noalloc_scratch(dev, &scratch);
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
    a.nsave_cap = (int)save_cap(o);
    a.save_everystep = o->save_everystep;
    a.callback = o->callback ? 1 : 0;
    a.interp_points = o->interp_points;
    a.tstops = o->ntstops > 0 ? o->tstops : nullptr;   // device memory, ascending
    a.ntstops = o->ntstops > 0 ? o->ntstops : 0;
    a.max_jac_age = o->max_jac_age;
    a.jac_reuse_gamma_tol = o->jac_reuse_gamma_tol < 0 ? 0.03 : o->jac_reuse_gamma_tol;
    a.adaptive = o->adaptive ? 1 : 0;
    a.forward_only = (o->forward_only && !o->force_dtmin && !o->isoutofdomain) ? 1 : 0;
    a.abstol_vec = o->abstol_vec;
    a.reltol_vec = o->reltol_vec;
    a.force_dtmin = o->force_dtmin ? 1 : 0;
    a.isoutofdomain = o->isoutofdomain;
    resolve_controller(a, d->alg_id, o);
    a.save_idxs = o->nsave_idxs > 0 ? o->save_idxs : nullptr;   // device memory at this point
    a.nsave_rows = o->nsave_idxs > 0 ? o->nsave_idxs : 0;
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
    e = cudaMemsetAsync(scratch, 0, kCounters * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return fail(nullptr, ODE_E_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    if (npt_dev == nullptr) {
        std::string why;
        const KernelVariant* v = variant_for(d, o->lanes_per_traj, &rc, &why);
        if (!v) return fail(nullptr, rc, why);
        return noalloc_launch(v, a, scratch, sm_count, s);
    }
    long long* order = (long long*)(scratch + kCounters);
    if (const FusedVariant* fv = find_fused(d->alg_id, d->model_id, d->precision)) {
        enqueue_bucketing(npt_dev, N, scratch, order, nsaved, retcode, s);
        a.order = order;
        e = launch_fused(fv, a, scratch, sm_count, s);
        if (e != cudaSuccess) return fail(nullptr, ODE_E_CUDA, std::string("launch ") + fv->name + ": " + cudaGetErrorString(e));
        return ODE_OK;
    }
    // one kernel per size class: the counts first, a kernel for every class
    // present, and only then the scatter (which writes the outputs of
    // trajectories of no class) and the launches
    enqueue_count(npt_dev, N, scratch, s);
    unsigned long long hc[kNumClasses + 1] = {0};
    e = cudaMemcpyAsync(hc, scratch + kOffCounts, sizeof(hc), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(nullptr, ODE_E_CUDA, std::string("bucket counts: ") + cudaGetErrorString(e));
    const KernelVariant* vk[kNumClasses];
    if ((rc = class_kernels(nullptr, d, hc, vk))) return rc;
    enqueue_scatter(npt_dev, N, scratch, order, nsaved, retcode, s);
    a.order = order;
    unsigned long long off[kNumClasses] = {0};
    unsigned long long acc = 0;
    for (int k = 0; k < kNumClasses; ++k) { off[k] = acc; acc += hc[k]; }
    for (int k = 0; k < kNumClasses; ++k) {
        if (hc[k] == 0) continue;
        EnsembleArgs ac = a;
        ac.order = order + off[k];
        ac.count = (long long)hc[k];
        rc = noalloc_launch(vk[k], ac, scratch + kOffClassQ + k, sm_count, s);
        if (rc) return rc;
    }
    return ODE_OK;
}
