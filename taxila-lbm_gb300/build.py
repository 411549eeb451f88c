"""Build libtaxila_gb300.so (sm_103a) in-tree with nvcc.

Every translation unit under csrc/ is compiled in parallel; the units that
hold the reference-order (exact) kernels get --fmad=false so that no
multiply-add is contracted.  Objects go to _build/, the library next to this
file.  Rebuilds only what changed.
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtaxila_gb300.so")
# arithmetic-pipe throughput probes (measurement only, not part of the C ABI)
PEAKS_SRC = os.path.join(CSRC, "peaks", "tx_peaks.cu")
PEAKS_LIB = os.path.join(HERE, "libtx_peaks.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr", "-I" + INCLUDE]
# extra nvcc options (e.g. -DTX_FLOAT_MIN_BLOCKS=2 to retune the float kernels'
# occupancy); a change of this value rebuilds every object
EXTRA = os.environ.get("TX_NVCC_EXTRA", "").split()


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _deps():
    return [p for p in glob.glob(os.path.join(CSRC, "*")) if p.endswith((".cuh", ".h"))] + \
        [os.path.join(INCLUDE, "taxila_gb300.h")]


def _compile(src, extra, stamp):
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    newest_dep = max(os.path.getmtime(p) for p in _deps() + [src, stamp])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj, None
    cmd = [_nvcc()] + ARCH + FLAGS + EXTRA + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, "%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr)
    return obj, None


def build(verbose=True, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "extra_flags.txt")
    want = " ".join(EXTRA)
    if not os.path.exists(stamp) or open(stamp).read() != want:
        with open(stamp, "w") as fh:
            fh.write(want)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    jobs = jobs or max(1, os.cpu_count() or 1)
    objs, errors = [], []
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = {ex.submit(_compile, s, ["--fmad=false"] if "_exact_" in os.path.basename(s) else [], stamp): s for s in srcs}
        for fut in cf.as_completed(futs):
            obj, err = fut.result()
            objs.append(obj)
            if err:
                errors.append(err)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n\n".join(errors))
    objs.sort()
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        subprocess.run(cmd, check=True)
    if not os.path.exists(PEAKS_LIB) or os.path.getmtime(PEAKS_LIB) < os.path.getmtime(PEAKS_SRC):
        cmd = [_nvcc()] + ARCH + ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", PEAKS_SRC, "-o", PEAKS_LIB]
        subprocess.run(cmd, check=True)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(jobs=int(sys.argv[1]) if len(sys.argv) > 1 else None)
