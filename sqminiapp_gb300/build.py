"""Build the in-tree shared library sqminiapp_gb300/lib/libsq_gb300.so with nvcc (sm_103a).

Translation units compile in parallel; quadrature.cu is compiled with -fmad=false so the
implicit-QL arithmetic is IEEE multiply/add exactly as in the CPU formulation.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "libsq_gb300.so")
DRIVER = os.path.join(LIB_DIR, "sq_lsdft")  # the command-line program (csrc/driver.cpp)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_LIB = "/usr/local/cuda/lib64"
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2", "-I", CSRC,
          "-I", os.path.join(os.path.dirname(HERE), "include")]
SOURCES = {
    "lanczos.cu": [],
    "lanczos_f32.cu": ["-Xptxas", "-v"],
    "lanczos_f32w.cu": ["-Xptxas", "-v"],
    "lanczos_f32n.cu": ["-Xptxas", "-v"],
    "lanczos_f32c.cu": ["-Xptxas", "-v"],
    "lanczos_f32q.cu": ["-Xptxas", "-v"],
    "lanczos_f32p.cu": ["-Xptxas", "-v"],
    "lanczos_f64.cu": ["-Xptxas", "-v"],
    "lanczos_f64x.cu": ["-Xptxas", "-v"],
    "quadrature.cu": ["-fmad=false"],
    "fermi.cu": [],
    "probe.cu": [],
    "capi.cpp": ["-x", "cu"],
    "setup.cpp": [],
    "deck.cpp": [],
    "scf_setup.cpp": [],
    "scf.cu": [],
    "io.cpp": [],
    "mlp.cu": ["-Xptxas", "-v"],
}


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _compile(src, extra, verbose):
    out = os.path.join(OBJ, src + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".hpp", ".cuh"))]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "sq_gb300.h"))
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out, ""
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", path, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return out, r.stderr if verbose else ""


def build(verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        futs = [ex.submit(_compile, s, e, verbose) for s, e in SOURCES.items()]
        objs = []
        for f in futs:
            o, log = f.result()
            objs.append(o)
            if log:
                sys.stderr.write(log)
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcufft", "-lcudart_static", "-lrt", "-ldl", "-lpthread",
                                                         "-Xlinker", "--no-undefined",
                                                         "-Xlinker", "-rpath=" + CUDA_LIB]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    src = os.path.join(CSRC, "driver.cpp")
    if (not os.path.exists(DRIVER) or os.path.getmtime(DRIVER) < os.path.getmtime(LIB) or
            os.path.getmtime(DRIVER) < os.path.getmtime(src)):
        cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(os.path.dirname(HERE), "include"),
               src, "-o", DRIVER, "-L", LIB_DIR, "-lsq_gb300", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("driver build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
