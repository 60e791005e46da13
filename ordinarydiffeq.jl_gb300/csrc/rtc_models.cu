// Models registered at run time (ode_register_model).
//
// The reference integrates any Julia f(du, u, p, t), with an optional analytic
// jac and tgrad (ODEFunction; the solve enters through lib/DiffEqBase/src/
// solve.jl:155-192).  Device code cannot call a Julia closure, so a caller
// registers the right-hand side as CUDA C++ source instead (the device form of
// the same function): the library compiles it with NVRTC together with the
// integrator templates (the headers are embedded in the library when it is
// built) into one kernel per (method, precision), loads the cubin with
// cudaLibraryLoadData and launches it through cudaLaunchKernel exactly like a
// compiled-in variant.  Kernels are compiled on the first solve that needs them
// (1-4 s each) and kept for the life of the process.  NVRTC is loaded with
// dlopen on the first registration, so the library has no link-time
// dependency on it.
#include "ode_gb300.h"
#include "ode_kernels.h"
#include "rtc_models.h"

#include <dlfcn.h>
#include <nvrtc.h>

#include <type_traits>

#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#ifndef ODEGB_NVRTC_PATH
#define ODEGB_NVRTC_PATH "libnvrtc.so"
#endif

namespace odegb {

// the integrator headers, embedded by the build (lib/obj/rtc_headers.cpp)
extern const char* const kRtcHeaderNames[];
extern const char* const kRtcHeaderSources[];
extern const int kRtcNumHeaders;

namespace {

struct Nvrtc {
    void* so = nullptr;
    const char* (*GetErrorString)(nvrtcResult) = nullptr;
    nvrtcResult (*CreateProgram)(nvrtcProgram*, const char*, const char*, int, const char* const*,
                                 const char* const*) = nullptr;
    nvrtcResult (*DestroyProgram)(nvrtcProgram*) = nullptr;
    nvrtcResult (*CompileProgram)(nvrtcProgram, int, const char* const*) = nullptr;
    nvrtcResult (*AddNameExpression)(nvrtcProgram, const char*) = nullptr;
    nvrtcResult (*GetLoweredName)(nvrtcProgram, const char*, const char**) = nullptr;
    nvrtcResult (*GetProgramLogSize)(nvrtcProgram, size_t*) = nullptr;
    nvrtcResult (*GetProgramLog)(nvrtcProgram, char*) = nullptr;
    nvrtcResult (*GetCUBINSize)(nvrtcProgram, size_t*) = nullptr;
    nvrtcResult (*GetCUBIN)(nvrtcProgram, char*) = nullptr;

    bool load(std::string* err) {
        if (so) return true;
        const char* cands[] = {ODEGB_NVRTC_PATH, "libnvrtc.so.13", "libnvrtc.so"};
        for (const char* c : cands)
            if ((so = dlopen(c, RTLD_NOW | RTLD_LOCAL)) != nullptr) break;
        if (!so) {
            *err = "NVRTC (libnvrtc.so) could not be loaded; registered models need the CUDA toolkit's NVRTC";
            return false;
        }
        bool ok = true;
        auto sym = [&](auto& fn, const char* name) {
            fn = reinterpret_cast<std::remove_reference_t<decltype(fn)>>(dlsym(so, name));
            ok = ok && fn != nullptr;
        };
        sym(GetErrorString, "nvrtcGetErrorString");
        sym(CreateProgram, "nvrtcCreateProgram");
        sym(DestroyProgram, "nvrtcDestroyProgram");
        sym(CompileProgram, "nvrtcCompileProgram");
        sym(AddNameExpression, "nvrtcAddNameExpression");
        sym(GetLoweredName, "nvrtcGetLoweredName");
        sym(GetProgramLogSize, "nvrtcGetProgramLogSize");
        sym(GetProgramLog, "nvrtcGetProgramLog");
        sym(GetCUBINSize, "nvrtcGetCUBINSize");
        sym(GetCUBIN, "nvrtcGetCUBIN");
        if (!ok) {
            *err = "libnvrtc.so lacks an entry point this library uses";
            dlclose(so);
            so = nullptr;
        }
        return ok;
    }
};

struct Compiled {
    KernelVariant v;
    std::string name;
    cudaLibrary_t lib = nullptr;
};

struct Registered {
    int id = 0, n = 0, np = 0, flags = 0;
    std::string name, source;
    std::map<std::pair<int, int>, std::unique_ptr<Compiled>> kernels;   // (alg, precision)
    std::map<std::pair<int, int>, std::string> failed;                  // compile errors, kept
};

std::mutex g_mu;
Nvrtc g_nvrtc;
std::vector<std::unique_ptr<Registered>> g_models;

bool valid_identifier(const char* s) {
    if (!s || !*s) return false;
    if (!((*s >= 'a' && *s <= 'z') || (*s >= 'A' && *s <= 'Z') || *s == '_')) return false;
    for (const char* c = s; *c; ++c)
        if (!((*c >= 'a' && *c <= 'z') || (*c >= 'A' && *c <= 'Z') || (*c >= '0' && *c <= '9') || *c == '_'))
            return false;
    return std::strlen(s) < 64;
}

const char* alg_type(int alg) {
    switch (alg) {
    case ODE_TSIT5: return "odegb::Tsit5Alg";
    case ODE_VERN7: return "odegb::Vern7Alg";
    case ODE_RODAS5P: return "odegb::Rodas5PAlg";
    case ODE_ROSENBROCK23: return "odegb::Rosenbrock23Alg";
    case ODE_AUTOTSIT5_ROSENBROCK23: return "odegb::AutoTsit5Rosenbrock23Alg";
    }
    return nullptr;
}
bool uses_jacobian(int alg) { return alg == ODE_RODAS5P || alg == ODE_ROSENBROCK23 || alg == ODE_AUTOTSIT5_ROSENBROCK23; }

// The program NVRTC compiles: the integrator headers, the caller's source, and
// the model adapter (the concept the kernel templates take: NP, AUTONOMOUS,
// rhs, jac, tgrad) around the caller's NAME_f / NAME_jac / NAME_tgrad.
std::string program(const Registered& m) {
    const std::string& N = m.name;
    const bool jac = m.flags & ODE_MODEL_HAS_JAC, tg = m.flags & ODE_MODEL_HAS_TGRAD;
    const bool nonauto = m.flags & ODE_MODEL_NONAUTONOMOUS;
    const bool ccb = m.flags & ODE_MODEL_CONTINUOUS_CALLBACK, vcb = m.flags & ODE_MODEL_VECTOR_CALLBACK;
    const bool dcb = m.flags & ODE_MODEL_DISCRETE_CALLBACK;
    const int vlen = (m.flags >> 16) & 0xff;
    std::string s;
    s += "#include \"erk.cuh\"\n#include \"rodas.cuh\"\n#include \"ros23.cuh\"\n#include \"autoswitch.cuh\"\n"
         "#include \"user_model.cuh\"\n";
    s += "#line 1 \"" + N + "\"\n" + m.source + "\n";
    s += "namespace odegb_user {\n";
    s += "struct f_of_" + N + " {\n  template <class T, class P> __device__ void operator()(T* du, const T* u, "
         "const P* p, double t) const { " + N + "_f(du, u, p, t); }\n};\n";
    s += "struct Model {\n";
    s += "  static constexpr int NP = " + std::to_string(m.np) + ";\n";
    s += std::string("  static constexpr bool AUTONOMOUS = ") + (nonauto ? "false" : "true") + ";\n";
    s += std::string("  static constexpr bool HAS_EVENT = ") + (ccb || vcb ? "true" : "false") + ";\n";
    s += "  static constexpr int EVENT_LEN = " + std::to_string(vcb ? vlen : 1) + ";\n";
    s += std::string("  static constexpr bool EVENT_AFFECT_POS = ") +
         (m.flags & ODE_MODEL_CALLBACK_AFFECT ? "true" : "false") + ";\n";
    s += std::string("  static constexpr bool EVENT_AFFECT_NEG = ") +
         (m.flags & ODE_MODEL_CALLBACK_AFFECT_NEG ? "true" : "false") + ";\n";
    s += std::string("  static constexpr bool HAS_DISCRETE = ") + (dcb ? "true" : "false") + ";\n";
    s += "  static constexpr bool DISCRETE_AT_TSTOPS = false;\n";
    // the callbacks see the state as FP64 (the pair hi + lo in the mixed form) and the
    // parameters as FP64, and write the state back as a pair
    s += "  template <class R, int C> __device__ static void gather(double* ud, double* pd, const R* u, "
         "const R* ulo, const double* p, long long stride) {\n"
         "    for (int c = 0; c < C; ++c) ud[c] = (double)u[c] + (double)ulo[c];\n"
         "    for (int i = 0; i < NP; ++i) pd[i] = p[(long long)i * stride];\n  }\n";
    s += "  template <class R, int C> __device__ static void scatter(R* u, R* ulo, const double* ud) {\n"
         "    for (int c = 0; c < C; ++c) odegb::Acc<R>::split(ud[c], u[c], ulo[c]);\n  }\n";
    const std::string args = "(const R* u, const R* ulo, const double* p, long long stride, double t, "
                             "const odegb::Group<L>&)";
    const std::string margs = "(R* u, R* ulo, const double* p, long long stride, double t, ";
    const std::string locals = "double ud[C], pd[NP > 0 ? NP : 1]; gather<R, C>(ud, pd, u, ulo, p, stride); ";
    if (ccb) {
        s += "  template <class R, int L, int C> __device__ static double event_condition" + args + " { " + locals +
             "return " + N + "_condition(ud, pd, t); }\n";
        s += "  template <class R, int L, int C> __device__ static bool event_affect" + margs +
             "bool up, const odegb::Group<L>&) { " + locals + "const int r = " + N +
             "_affect(ud, pd, t, up ? 1 : 0); scatter<R, C>(u, ulo, ud); return r != 0; }\n";
    }
    if (vcb) {
        s += "  template <class R, int L, int C> __device__ static void event_conditions(double* out, const R* u, "
             "const R* ulo, const double* p, long long stride, double t, const odegb::Group<L>&) { " + locals +
             N + "_vcondition(out, ud, pd, t); }\n";
        s += "  template <class R, int L, int C> __device__ static bool vector_event_affect" + margs +
             "const int* events, const odegb::Group<L>&) { " + locals + "const int r = " + N +
             "_vaffect(ud, pd, t, events); scatter<R, C>(u, ulo, ud); return r != 0; }\n";
    }
    if (dcb) {
        s += "  template <class R, int L, int C> __device__ static bool discrete_condition" + args + " { " + locals +
             "return " + N + "_dcondition(ud, pd, t) != 0; }\n";
        s += "  template <class R, int L, int C> __device__ static bool discrete_affect" + margs +
             "const odegb::Group<L>&) { " + locals + "const int r = " + N +
             "_daffect(ud, pd, t); scatter<R, C>(u, ulo, ud); return r != 0; }\n";
    }
    s += std::string("  static constexpr bool HAS_TGRAD = ") + (tg ? "true" : "false") + ";\n";
    s += std::string("  static constexpr int JAC_F_CALLS = ") + (jac ? "0" : "1") + ";\n";
    s += "  template <class R, int L, int C, class P>\n  __device__ static void rhs(R* du, const R* u, const P* p, "
         "double t, const odegb::Group<L>&) { " + N + "_f(du, u, p, t); }\n";
    s += "  template <class R, int NN, class P>\n  __device__ static void jac(R (*J)[NN], const R* u, const P* p, "
         "double t) { ";
    s += jac ? N + "_jac(&J[0][0], u, p, t); }\n" : "odegb::ad_jacobian<R, NN>(f_of_" + N + "(), J, u, p, t); }\n";
    if (tg)
        s += "  template <class R, int C, class P>\n  __device__ static void tgrad(R* dT, const R* u, const P* p, "
             "double t) { " + N + "_tgrad(dT, u, p, t); }\n";
    s += "};\n}  // namespace odegb_user\n";
    return s;
}

int compile(Registered& m, int alg, int prec, Compiled* out, std::string* err) {
    if (!g_nvrtc.load(err)) return ODE_E_UNSUPPORTED;
    int dev = 0, major = 0, minor = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (e != cudaSuccess) {
        *err = std::string("device query: ") + cudaGetErrorString(e);
        return ODE_E_CUDA;
    }
    char arch[48];
    std::snprintf(arch, sizeof arch, "--gpu-architecture=sm_%d%d%s", major, minor, major >= 9 ? "a" : "");
    const std::string src = program(m);
    const std::string expr = std::string("odegb::ensemble_kernel<") + alg_type(alg) + ", odegb_user::Model, " +
                             (prec == ODE_PREC_FP64 ? "double" : "float") + ", 1, " + std::to_string(m.n) + ">";
    nvrtcProgram prog = nullptr;
    nvrtcResult r = g_nvrtc.CreateProgram(&prog, src.c_str(), (m.name + ".cu").c_str(), kRtcNumHeaders,
                                          kRtcHeaderSources, kRtcHeaderNames);
    if (r != NVRTC_SUCCESS) {
        *err = std::string("nvrtcCreateProgram: ") + g_nvrtc.GetErrorString(r);
        return ODE_E_UNSUPPORTED;
    }
    g_nvrtc.AddNameExpression(prog, expr.c_str());
    // the compiled-in kernels' flags: every multiply-add written out (-fmad=false)
    const char* opts[] = {arch, "-std=c++17", "--fmad=false", "-default-device", "-diag-suppress=128"};
    r = g_nvrtc.CompileProgram(prog, (int)(sizeof(opts) / sizeof(opts[0])), opts);
    if (r != NVRTC_SUCCESS) {
        size_t n = 0;
        g_nvrtc.GetProgramLogSize(prog, &n);
        std::string log(n, '\0');
        if (n) g_nvrtc.GetProgramLog(prog, &log[0]);
        if (log.size() > 6000) log.resize(6000);
        *err = "compiling model '" + m.name + "' for " + alg_type(alg) + " failed:\n" + log;
        g_nvrtc.DestroyProgram(&prog);
        return ODE_E_UNSUPPORTED;
    }
    const char* lowered = nullptr;
    g_nvrtc.GetLoweredName(prog, expr.c_str(), &lowered);
    out->name = lowered ? lowered : "";
    size_t nbin = 0;
    g_nvrtc.GetCUBINSize(prog, &nbin);
    std::vector<char> cubin(nbin);
    if (nbin) g_nvrtc.GetCUBIN(prog, cubin.data());
    g_nvrtc.DestroyProgram(&prog);
    if (out->name.empty() || nbin == 0) {
        *err = "NVRTC produced no kernel for model '" + m.name + "'";
        return ODE_E_UNSUPPORTED;
    }
    e = cudaLibraryLoadData(&out->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    cudaKernel_t k = nullptr;
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&k, out->lib, out->name.c_str());
    if (e != cudaSuccess) {
        *err = std::string("loading the compiled model: ") + cudaGetErrorString(e);
        return ODE_E_CUDA;
    }
    out->v.alg = alg;
    out->v.model = m.id;
    out->v.prec = prec;
    out->v.n = m.n;
    out->v.lanes = 1;
    out->v.smem_per_group = 0;
    out->v.fn = (const void*)k;
    out->v.launch = nullptr;   // launched by handle through cudaLaunchKernel
    out->name = m.name + "/" + alg_type(alg) + (prec == ODE_PREC_FP64 ? "/double" : "/float");
    out->v.name = out->name.c_str();
    return ODE_OK;
}

Registered* find(int id) {
    const int k = id - ODE_MODEL_USER_BASE;
    if (k < 0 || k >= (int)g_models.size()) return nullptr;
    return g_models[k].get();
}

}  // namespace

int rtc_register(const char* source, const char* name, int n, int np, int flags, int* id, std::string* err) {
    if (!source || !valid_identifier(name)) {
        *err = "a registered model needs its source and a C identifier as its name";
        return ODE_E_INVALID;
    }
    if (n < 1 || n > kRtcMaxStates || np < 0 || np > kRtcMaxParams) {
        char buf[128];
        std::snprintf(buf, sizeof buf, "registered models take 1..%d states and 0..%d parameters", kRtcMaxStates,
                      kRtcMaxParams);
        *err = buf;
        return ODE_E_INVALID;
    }
    const int known = ODE_MODEL_HAS_JAC | ODE_MODEL_HAS_TGRAD | ODE_MODEL_NONAUTONOMOUS |
                      ODE_MODEL_CONTINUOUS_CALLBACK | ODE_MODEL_CALLBACK_AFFECT | ODE_MODEL_CALLBACK_AFFECT_NEG |
                      ODE_MODEL_VECTOR_CALLBACK | ODE_MODEL_DISCRETE_CALLBACK | ODE_MODEL_CALLBACK_LEN(0xff);
    if (flags & ~known) {
        *err = "unknown model flag";
        return ODE_E_INVALID;
    }
    const int vlen = (flags >> 16) & 0xff;
    if ((flags & ODE_MODEL_CONTINUOUS_CALLBACK) && (flags & ODE_MODEL_VECTOR_CALLBACK)) {
        *err = "a model registers one continuous callback: scalar or vector";
        return ODE_E_INVALID;
    }
    if ((flags & ODE_MODEL_CONTINUOUS_CALLBACK) &&
        !(flags & (ODE_MODEL_CALLBACK_AFFECT | ODE_MODEL_CALLBACK_AFFECT_NEG))) {
        *err = "a ContinuousCallback needs affect! (ODE_MODEL_CALLBACK_AFFECT) or affect_neg! "
               "(ODE_MODEL_CALLBACK_AFFECT_NEG)";
        return ODE_E_INVALID;
    }
    if ((flags & ODE_MODEL_VECTOR_CALLBACK) ? (vlen < 1 || vlen > 32) : vlen != 0) {
        *err = "a VectorContinuousCallback takes ODE_MODEL_CALLBACK_LEN(len) with 1 <= len <= 32, and only it";
        return ODE_E_INVALID;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_nvrtc.load(err)) return ODE_E_UNSUPPORTED;
    auto m = std::make_unique<Registered>();
    m->id = ODE_MODEL_USER_BASE + (int)g_models.size();
    m->n = n;
    m->np = np;
    m->flags = flags;
    m->name = name;
    m->source = source;
    *id = m->id;
    g_models.push_back(std::move(m));
    return ODE_OK;
}

bool rtc_lookup(int model, int* n, int* np, int* flags) {
    std::lock_guard<std::mutex> lk(g_mu);
    const Registered* m = find(model);
    if (!m) return false;
    if (n) *n = m->n;
    if (np) *np = m->np;
    if (flags) *flags = m->flags;
    return true;
}

const KernelVariant* rtc_variant(int alg, int model, int prec, int* status, std::string* err) {
    std::lock_guard<std::mutex> lk(g_mu);
    Registered* m = find(model);
    *status = ODE_OK;
    if (!m) {
        *status = ODE_E_INVALID;
        *err = "unknown model_id";
        return nullptr;
    }
    if (!alg_type(alg)) {
        *status = ODE_E_INVALID;
        *err = "unknown alg_id";
        return nullptr;
    }
    if (uses_jacobian(alg) && m->n > kRtcMaxStatesRosenbrock) {
        *status = ODE_E_UNSUPPORTED;
        char buf[160];
        std::snprintf(buf, sizeof buf, "registered models solved by a Rosenbrock method take at most %d states "
                      "(W and its LU live in registers)", kRtcMaxStatesRosenbrock);
        *err = buf;
        return nullptr;
    }
    if (uses_jacobian(alg) && (m->flags & ODE_MODEL_NONAUTONOMOUS) && !(m->flags & ODE_MODEL_HAS_TGRAD)) {
        *status = ODE_E_UNSUPPORTED;
        *err = "a non-autonomous model solved by a Rosenbrock method needs its time derivative (" + m->name +
               "_tgrad, ODE_MODEL_HAS_TGRAD)";
        return nullptr;
    }
    const auto key = std::make_pair(alg, prec);
    auto it = m->kernels.find(key);
    if (it != m->kernels.end()) return &it->second->v;
    auto f = m->failed.find(key);
    if (f != m->failed.end()) {
        *status = ODE_E_UNSUPPORTED;
        *err = f->second;
        return nullptr;
    }
    auto c = std::make_unique<Compiled>();
    const int rc = compile(*m, alg, prec, c.get(), err);
    if (rc != ODE_OK) {
        *status = rc;
        if (rc == ODE_E_UNSUPPORTED) m->failed[key] = *err;
        return nullptr;
    }
    const KernelVariant* v = &c->v;
    m->kernels[key] = std::move(c);
    return v;
}

}  // namespace odegb
