"""Build libode_b200.so (sm_103a) in-tree with nvcc.

Translation units compile in parallel; the library is rebuilt only when a
source or header is newer than it.  Output: ordinarydiffeq.jl_gb300/lib/.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(PKG, "lib")
OBJ_DIR = os.path.join(PKG, "lib", "obj")
LIB_PATH = os.path.join(OUT_DIR, "libode_b200.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: kernels spell out every fused multiply-add (reference op order).
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


# Device headers embedded in the library for the run-time compilation of
# registered models (NVRTC compiles them with the caller's source).
RTC_HEADERS = ["common.cuh", "ensemble_args.h", "integrator.cuh", "rksum.cuh", "tableaus.h", "erk.cuh",
               "lu_group.cuh", "rodas.cuh", "ros23.cuh", "autoswitch.cuh", "user_model.cuh"]
_RAW = "ODEGBRTC"


def write_rtc_headers(path):
    """A C++ source holding every RTC header's text as a raw string literal."""
    names, texts = [], []
    for h in RTC_HEADERS:
        text = open(os.path.join(CSRC, h)).read()
        if (")" + _RAW + '"') in text:
            raise RuntimeError("header %s contains the raw-string delimiter" % h)
        names.append(h)
        texts.append(text)
    out = ["// Generated by odegb300/build.py: the device headers, for NVRTC.", "namespace odegb {",
           "extern const char* const kRtcHeaderNames[] = {" + ", ".join('"%s"' % n for n in names) + "};",
           "extern const char* const kRtcHeaderSources[] = {"]
    for t in texts:
        out.append('R"%s(%s)%s",' % (_RAW, t, _RAW))
    out += ["};", "extern const int kRtcNumHeaders = %d;" % len(names), "}  // namespace odegb", ""]
    with open(path, "w") as fh:
        fh.write("\n".join(out))


def nvrtc_path():
    cand = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))), "lib64", "libnvrtc.so")
    return cand if os.path.exists(cand) else "libnvrtc.so"


def _deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h")) + [os.path.abspath(__file__)]


def up_to_date():
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(p) <= t for p in _deps())


def _compile(src, verbose):
    obj = os.path.join(OBJ_DIR, os.path.splitext(os.path.basename(src))[0] + ".o")
    # ODEGB_EXTRA_NVCC_FLAGS: tuning defines, e.g. -DODEGB_MIN_BLOCKS_F32=4
    extra = os.environ.get("ODEGB_EXTRA_NVCC_FLAGS", "").split()
    if os.path.basename(src) == "rtc_models.cu":
        extra = extra + ['-DODEGB_NVRTC_PATH="%s"' % nvrtc_path()]
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-6000:]))
    return obj, r.stderr


def build(force=False, verbose=False, jobs=None):
    """Compile every CUDA translation unit for sm_103a and link the library."""
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(OBJ_DIR, exist_ok=True)
    rtc = os.path.join(OBJ_DIR, "rtc_headers.cpp")
    write_rtc_headers(rtc)
    srcs = sources() + [rtc]
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    logs = {}
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = {ex.submit(_compile, s, verbose): s for s in srcs}
        objs = []
        for f in cf.as_completed(futs):
            obj, log = f.result()
            objs.append(obj)
            logs[futs[f]] = log
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + sorted(objs) + ["-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    os.replace(tmp, LIB_PATH)
    if verbose:
        for k, v in logs.items():
            print("==", os.path.basename(k))
            print(v)
    return LIB_PATH


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
