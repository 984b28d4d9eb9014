"""In-tree build of the GB300 library (libsflow_gb300.so).

nvcc compiles the CUDA translation units for sm_103a only; the FP64 plain
form is compiled with --fmad=false so that its arithmetic follows the
reference operation order; the FP32 bulk form with fused multiply-add,
flush-to-zero and the approximate (<= 2 ulp) single-precision division and
square root (its FP64 Newton step and sums are unaffected).  The host set-up and the C ABI are plain C++.
Translation units compile in parallel; the library links the CUDA runtime
statically so it loads without a torch or CUDA toolkit environment.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(HERE, "..", "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsflow_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

FP64 = ["--fmad=false"]
FP32 = ["--fmad=true", "-ftz=true", "-prec-div=false", "-prec-sqrt=false"]
UNITS = [
    # (source, extra flags); the class-count / tile-height kernels are the
    # slow units and start first
    ("sflow_k_fp64_ns2.cu", FP64),
    ("sflow_k_fp32_ns2.cu", FP32),
    ("sflow_k_fp32_ns2_t16.cu", FP32),
    ("sflow_k_fp32_ns2_t4.cu", FP32),
    ("sflow_k_fp64_ns3.cu", FP64),
    ("sflow_k_fp32_ns3.cu", FP32),
    ("sflow_k_fp32_ns3_t16.cu", FP32),
    ("sflow_k_fp32_ns3_t4.cu", FP32),
    ("sflow_k_fp64_ns1.cu", FP64),
    ("sflow_k_fp32_ns1.cu", FP32),
    ("sflow_k_fp32_ns1_t16.cu", FP32),
    ("sflow_k_fp32_ns1_t4.cu", FP32),
    ("sflow_noalloc.cu", FP64),
    ("sflow_fp64.cu", FP64),
    ("sflow_fp32.cu", FP32),
    ("sflow_setup.cpp", []),
    ("sflow_capi.cpp", []),
    ("sflow_io.cpp", []),
]


def _nvcc():
    for c in ("/usr/local/cuda/bin/nvcc", "nvcc"):
        if os.path.exists(c) or c == "nvcc":
            return c
    return "nvcc"


def _sources():
    out = []
    for f in os.listdir(CSRC):
        out.append(os.path.join(CSRC, f))
    out.append(os.path.join(INC, "sflow.h"))
    return out


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _sources())


def build(force=False, verbose=False, ptxas_verbose=False):
    """Compile and link libsflow_gb300.so if any source is newer."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    procs = []
    objs = []
    for src, extra in UNITS:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        path = os.path.join(CSRC, src)
        if src.endswith(".cu"):
            cmd = [nvcc, "-c", path, "-o", obj, "-std=c++17", "-O3", "-lineinfo",
                   "-Xcompiler", "-fPIC", "-I", INC, "--expt-relaxed-constexpr"] + ARCH + extra
            if ptxas_verbose:
                cmd += ["-Xptxas", "-v"]
        else:
            cmd = ["g++", "-c", path, "-o", obj, "-std=c++17", "-O2", "-fPIC", "-Wall",
                   "-ffp-contract=off", "-I", INC]
        if verbose:
            print(" ".join(cmd))
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        text = out.decode(errors="replace")
        if p.returncode != 0:
            failed.append((src, text))
        elif verbose or ptxas_verbose:
            if text.strip():
                print(text)
    if failed:
        msg = "\n".join(f"--- {s}\n{t}" for s, t in failed)
        raise RuntimeError("libsflow_gb300 build failed:\n" + msg)
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-shared", "-o", tmp] + objs + ["-cudart", "static"] + ARCH
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                ptxas_verbose="--ptxas" in sys.argv))
