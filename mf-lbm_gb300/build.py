"""Build libmflbm.so (sm_103a) in-tree.

The translation units are compiled in parallel and linked into
mf-lbm_gb300/mflbm/lib/libmflbm.so:

  csrc/api.cu             C ABI, context, step ordering, CUDA graphs
  csrc/kernels_fast*.cu   kernels with nvcc's default FMA contraction, in three units
                          (collision sweeps; ensembles; the rest and the launch table)
  csrc/kernels_strict*.cu the same kernels with --fmad=false (bit-identical to an IEEE
                          restatement that keeps the reference's operation order)
  csrc/noalloc.cu         mflbm_saturation_noalloc (fixed device scratch, no allocation)
  csrc/listlayout.cpp     host construction of the fluid-list layout
  csrc/ensemble.cu        batched samples in one fluid-list arena, launch-shape autotuner
  csrc/nn_gemm.cu         BF16 tcgen05 GEMM (TMEM accumulators) of the warm-start network
  csrc/nn_ops.cu          im2col/col2im, pooling, upsampling, loss and Adam of that network
  csrc/preprocess.cu      geometry_preprocessing_new on the GPU (boundary-node lists)

Only one -gencode (sm_103a) is built.  nvcc cross-compiles without a GPU, so this runs
on the CPU build host and on the GPU host alike.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "mflbm", "lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmflbm.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "--expt-relaxed-constexpr"]
# extra nvcc flags for tuning builds (e.g. MFLBM_NVCC_FLAGS="-DMFLBM_FF_MIN_BLOCKS=5")
EXTRA = os.environ.get("MFLBM_NVCC_FLAGS", "").split()
UNITS = {
    "api.o": ("api.cu", []),
    "kernels_fast_sweep.o": ("kernels_fast_sweep.cu", []),
    "kernels_fast_ens.o": ("kernels_fast_ens.cu", []),
    "kernels_fast.o": ("kernels_fast.cu", []),
    "kernels_strict_sweep.o": ("kernels_strict_sweep.cu", ["--fmad=false"]),
    "kernels_strict_ens.o": ("kernels_strict_ens.cu", ["--fmad=false"]),
    "kernels_strict.o": ("kernels_strict.cu", ["--fmad=false"]),
    "noalloc.o": ("noalloc.cu", []),
    "listlayout.o": ("listlayout.cpp", []),
    "ensemble.o": ("ensemble.cu", []),
    "nn_gemm.o": ("nn_gemm.cu", []),
    "nn_ops.o": ("nn_ops.cu", []),
    "preprocess.o": ("preprocess.cu", []),
}


def nvcc():
    exe = shutil.which("nvcc")
    if exe is None:
        cand = "/usr/local/cuda/bin/nvcc"
        if os.path.exists(cand):
            return cand
        raise RuntimeError("nvcc not found")
    return exe


def _sources_mtime():
    m = 0.0
    for root in (CSRC, os.path.join(HERE, "..", "include")):
        for name in os.listdir(root):
            m = max(m, os.path.getmtime(os.path.join(root, name)))
    return m


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime():
        return LIB
    exe = nvcc()
    procs = []
    for obj, (src, extra) in UNITS.items():
        cmd = [exe, *ARCH, *COMMON, *extra, *EXTRA, "-c", os.path.join(CSRC, src), "-o", os.path.join(BUILD_DIR, obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((subprocess.Popen(cmd), obj))
    failed = [obj for p, obj in procs if p.wait() != 0]
    if failed:
        raise RuntimeError(f"nvcc failed for {failed}")
    tmp = LIB + ".tmp"
    cmd = [exe, *ARCH, "-shared", "-o", tmp, *[os.path.join(BUILD_DIR, o) for o in UNITS]]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
