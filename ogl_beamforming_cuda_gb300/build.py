"""Build lib/libogl_beamformer_lib.so in tree (sm_103a kernels + C++ host code).

nvcc compiles each CUDA translation unit for sm_103a only; g++ compiles the host
code; both with -ffp-contract=off on the host side (the voxel transform and the
constants of the DAS delay chain must round as the reference's expressions do).
Translation units compile in parallel; an unchanged object is not rebuilt.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libogl_beamformer_lib.so")
SERVER = os.path.join(LIBDIR, "ogl_beamformer_server")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INC = [f"-I{os.path.join(ROOT, 'include')}", f"-I{CSRC}"]

CU = ["bf_decode.cu", "bf_filter.cu", "bf_fir_tc.cu", "bf_das.cu", "bf_das_hercules.cu", "bf_das_forces.cu", "bf_das_batch.cu", "bf_reduce.cu", "bf_hilbert.cu", "bf_unet.cu", "bf_unet_tc.cu"]
CPP = ["bf_host.cpp", "bf_library.cpp", "bf_server.cpp"]
HEADERS = ["bf_kernels.h", "bf_host.h", "bf_das_math.cuh", "bf_das_generic.cuh", "bf_das_hercules.cuh", "bf_das_staged.cuh", "bf_das_forces.cuh"]


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "ogl_beamformer_lib.h"), os.path.join(ROOT, "include", "bf_unet.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose=False, ptxas_info=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    jobs = []
    for f in CU:
        src, obj = os.path.join(CSRC, f), os.path.join(OBJ, f + ".o")
        if _stale(obj, src) or ptxas_info:
            cmd = [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                                   "-Xcompiler", "-fPIC,-ffp-contract=off", "-c", src, "-o", obj] + INC
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for f in CPP:
        src, obj = os.path.join(CSRC, f), os.path.join(OBJ, f + ".o")
        if _stale(obj, src):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
                         "-fvisibility=hidden", f"-I{CUDA}/include", "-c", src, "-o", obj] + INC)
    out = []
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for o in ex.map(_run, jobs):
            out.append(o)
    objs = [os.path.join(OBJ, f + ".o") for f in CU + CPP]
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        _run([NVCC] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs +
             ["-Xlinker", f"-rpath={CUDA}/lib64"])
        os.replace(tmp, LIB)
    # the shared-memory server: a small executable on top of the library
    srv_src = os.path.join(CSRC, "bf_server_main.cpp")
    if not os.path.exists(SERVER) or os.path.getmtime(SERVER) < max(os.path.getmtime(srv_src), os.path.getmtime(LIB)):
        tmp = SERVER + ".tmp"
        _run(["g++", "-O2", "-std=c++17", "-Wall", srv_src, "-o", tmp] + INC +
             [f"-L{LIBDIR}", "-logl_beamformer_lib", "-Wl,-rpath,$ORIGIN", "-lpthread"])
        os.replace(tmp, SERVER)
    text = "".join(out)
    if verbose and text:
        print(text)
    return text


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
