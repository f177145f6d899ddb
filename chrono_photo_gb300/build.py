"""Builds libchrono_gpu.so (CUDA kernels for sm_103a + the C++ host layer) in-tree.

Translation units are compiled in parallel: the kernels once per supported channel count,
the host sources with the system C++ compiler, then linked by nvcc into
chrono_photo_gb300/lib/libchrono_gpu.so.
"""
import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(LIB_DIR, "libchrono_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no multiply-add contraction, every f32 op rounds like the reference's.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-O3",
              "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread"]

CU_SOURCES = ["cp_kernels_c3.cu", "cp_kernels_c4.cu", "cp_kernels_c1.cu", "cp_shake.cu",
              "cp_static.cu", "cp_video.cu", "cp_kernels_multi.cu"]
# cp_kernels_variant.cu compiled once per specialised single-stack outlier kernel:
# (channels, distance kind, outlier group, background), the CP_VARIANTS list of cp_internal.h
KERNEL_VARIANTS = [(3, k, g, b) for k in (1, 2) for b in (1, 0) for g in (1, 2, 3)] + \
    [(3, 3, 0, 0), (1, 1, 0, 0), (1, 2, 0, 0), (1, 3, 0, 0), (4, 1, 0, 0), (4, 2, 0, 0),
     (4, 3, 0, 0)]
# cp_kernels_batch_variant.cu: the CP_BATCH_VARIANTS list of cp_internal.h
BATCH_VARIANTS = [(3, k, g, 1) for k in (1, 2) for g in (1, 2, 3)]
# cp_kernels_px.cu compiled once per pixel-thread kernel family (distance kind, outlier
# group, background): the CP_PX_VARIANTS list of cp_internal.h
PX_VARIANTS = [(k, g, b) for k in (1, 2) for b in (1, 0) for g in (1, 2, 3)]
CPP_SOURCES = ["cp_host.cpp", "cp_prepare.cpp", "cp_memory.cpp", "cp_stage.cpp", "cp_batch.cpp",
               "cp_shake_host.cpp", "cp_server.cpp", "cp_ingest.cpp", "cp_png_write.cpp", "cp_tune.cpp",
               "cp_jpeg.cpp", "cp_jpeg_write.cpp"]
HEADERS = ["cp_internal.h", "cp_host_internal.h", "cp_tile.cuh", "cp_png.h", "cp_pixel.cuh",
           "cp_outlier_px.cuh", "cp_outlier_multi.cuh", "cp_io.h"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(c):
            return c
    nvcc = shutil.which("nvcc")
    return os.path.dirname(os.path.dirname(nvcc)) if nvcc else "/usr/local/cuda"


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def _arch_stamp():
    """Objects and the library built on another host architecture (a copied tree) are
    rebuilt: the stamp records the machine they were built for."""
    stamp = os.path.join(OBJ_DIR, "HOST_ARCH")
    here = platform.machine()
    try:
        same = open(stamp).read().strip() == here
    except OSError:
        same = False
    if not same:
        for d in (OBJ_DIR, LIB_DIR):
            for f in os.listdir(d):
                if f.endswith((".o", ".so", ".tmp")):
                    os.remove(os.path.join(d, f))
        with open(stamp, "w") as f:
            f.write(here + "\n")


def build(verbose=False, jobs=None):
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    cxx = os.environ.get("CXX", "g++")
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    _arch_stamp()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS]
    hdrs.append(os.path.join(HERE, "..", "include", "chrono_gpu.h"))
    steps, objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ_DIR, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            steps.append([nvcc] + ARCH + NVCC_FLAGS + ["-c", s, "-o", o])
    vsrc = os.path.join(CSRC, "cp_kernels_variant.cu")
    for ch, kind, og, bg in KERNEL_VARIANTS:
        o = os.path.join(OBJ_DIR, "cp_kernels_c%d_k%d_g%d_b%d.o" % (ch, kind, og, bg))
        objs.append(o)
        if _stale(o, [vsrc] + hdrs):
            steps.append([nvcc] + ARCH + NVCC_FLAGS + [
                "-DCP_CH=%d" % ch, "-DCP_KIND=%d" % kind, "-DCP_OG=%d" % og, "-DCP_BG=%d" % bg,
                "-c", vsrc, "-o", o])
    bsrc = os.path.join(CSRC, "cp_kernels_batch_variant.cu")
    for ch, kind, og, bg in BATCH_VARIANTS:
        o = os.path.join(OBJ_DIR, "cp_kernels_batch_c%d_k%d_g%d_b%d.o" % (ch, kind, og, bg))
        objs.append(o)
        if _stale(o, [bsrc] + hdrs):
            steps.append([nvcc] + ARCH + NVCC_FLAGS + [
                "-DCP_CH=%d" % ch, "-DCP_KIND=%d" % kind, "-DCP_OG=%d" % og, "-DCP_BG=%d" % bg,
                "-c", bsrc, "-o", o])
    psrc = os.path.join(CSRC, "cp_kernels_px.cu")
    for kind, og, bg in PX_VARIANTS:
        o = os.path.join(OBJ_DIR, "cp_kernels_px_k%d_g%d_b%d.o" % (kind, og, bg))
        objs.append(o)
        if _stale(o, [psrc] + hdrs):
            steps.append([nvcc] + ARCH + NVCC_FLAGS + [
                "-DCP_KIND=%d" % kind, "-DCP_OG=%d" % og, "-DCP_BG=%d" % bg,
                "-c", psrc, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ_DIR, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            steps.append([cxx] + CXX_FLAGS + ["-I", os.path.join(cuda, "include"), "-c", s, "-o", o])
    jobs = jobs or max(1, min(len(steps), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for out in ex.map(_run, steps):
            if verbose and out.strip():
                print(out)
    if steps or not os.path.exists(LIB_PATH):
        tmp = LIB_PATH + ".tmp"
        _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread", "-ldl"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
