"""Build ``libcomrs_gb300.so`` in-tree: CUDA sources for sm_103a, host C++ with g++.

``python -m``-free: ``python com-rs_gb300/build.py`` or ``build()`` from Python.
Translation units compile in parallel; the link is one nvcc call.
"""

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcomrs_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no multiply-add contraction, so every f64/f32 step rounds as the
# reference's separate operations do
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr"] + ARCH
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall"]

CU = ["decode.cu", "decode_nr.cu", "gen.cu", "nms_learned.cu", "mix.cu", "sparse.cu", "sparse_encode.cu", "link.cu", "nr_generic.cu", "capi.cu",
      "capi_mix.cu", "capi_sparse.cu"]
CPP = ["code_host.cpp", "sparse_host.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build comrs_gb300")


# the kernel source files the library compiles again at run time (NVRTC), embedded as text
JIT_FILES = ["dev_math.cuh", "nr_bg_schedule.inc", "layered_nr.cuh"]
JIT_INC = "nr_jit_sources.inc"


def _write_jit_sources(out_dir):
    """`<out_dir>/nr_jit_sources.inc`: the files of JIT_FILES as C++ raw string literals
    (rewritten only when their text changes, so that the object depending on it stays
    fresh otherwise)."""
    parts = ["// Generated by build.py: the decoder's kernel sources for the run-time compiler.\n",
             f"static const int kJitFileCount = {len(JIT_FILES)};\n",
             "static const char* const kJitFileNames[] = {" + ", ".join(f'"{f}"' for f in JIT_FILES) + "};\n",
             "static const char* const kJitFileTexts[] = {\n"]
    for f in JIT_FILES:
        text = open(os.path.join(CSRC, f)).read()
        if ")cbjit" in text:
            raise RuntimeError(f"{f} contains the raw-string delimiter")
        parts.append('R"cbjit(' + text + ')cbjit",\n')
    parts.append("};\n")
    body = "".join(parts)
    path = os.path.join(out_dir, JIT_INC)
    if not os.path.exists(path) or open(path).read() != body:
        with open(path, "w") as fh:
            fh.write(body)
    return path


def _stale(obj, deps):
    return not os.path.exists(obj) or any(os.path.getmtime(d) > os.path.getmtime(obj) for d in deps)


def build(verbose=False, extra_flags=(), out_dir=None, lib=None):
    """Compile (only stale objects) and link; out_dir/lib override the build paths."""
    OUT = out_dir or OUT_DIR
    LIBP = lib or LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".inc"))]
    headers.append(os.path.join(HERE, "..", "include", "comrs_gb300.h"))
    headers.append(_write_jit_sources(OUT))
    jobs = []
    for f in CU:
        src, obj = os.path.join(CSRC, f), os.path.join(OUT, f + ".o")
        if _stale(obj, [src] + headers):
            jobs.append([nvcc, *NVCC_FLAGS, *extra_flags, "-I", OUT, "-c", src, "-o", obj])
    for f in CPP:
        src, obj = os.path.join(CSRC, f), os.path.join(OUT, f + ".o")
        if _stale(obj, [src] + headers):
            jobs.append(["g++", *CXX_FLAGS, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError(f"compile failed: {os.path.basename(cmd[-3])}")
        return r

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(OUT, f + ".o") for f in CU + CPP]
    if jobs or not os.path.exists(LIBP):
        run([nvcc, *ARCH, "-shared", "-o", LIBP, *objs, "-lcudart", "-ldl"])
    return LIBP


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
