"""Build the host emulation binary (tests/hostemu/_build/emu) with g++.

The flow kernels of taxila-lbm_gb300/csrc/tx_kernels.cuh are compiled as
plain C++ against the stand-in headers in shim/, with AddressSanitizer and
UndefinedBehaviorSanitizer when the compiler has them, so that every index a
kernel forms is checked on the CPU.  Rebuilds only what changed.
"""
import concurrent.futures as cf
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
BUILD = os.path.join(HERE, "_build")
EXE = os.path.join(BUILD, "emu")
CSRC = os.path.join(REPO, "taxila-lbm_gb300", "csrc")
INCLUDE = os.path.join(REPO, "include")
SAN = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer"]
BASE = ["-std=c++17", "-O1", "-g", "-ffp-contract=off", "-I" + os.path.join(HERE, "shim"), "-I" + CSRC, "-I" + INCLUDE]


def _sanitizers_work(cxx):
    probe = os.path.join(BUILD, "probe.cpp")
    with open(probe, "w") as f:
        f.write("int main() { return 0; }\n")
    r = subprocess.run([cxx] + SAN + [probe, "-o", probe + ".bin"], capture_output=True)
    return r.returncode == 0


def _deps():
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) +
            glob.glob(os.path.join(HERE, "*.h")) + glob.glob(os.path.join(HERE, "shim", "*.h")) +
            [os.path.join(INCLUDE, "taxila_gb300.h")])


def build(cxx="g++"):
    os.makedirs(BUILD, exist_ok=True)
    flags = BASE + (SAN if _sanitizers_work(cxx) else [])
    srcs = sorted(glob.glob(os.path.join(HERE, "*.cpp")))
    stamp = os.path.join(BUILD, "flags.txt")
    if not os.path.exists(stamp) or open(stamp).read() != " ".join(flags):
        with open(stamp, "w") as f:
            f.write(" ".join(flags))
    dep_time = max(os.path.getmtime(p) for p in _deps() + [stamp])

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src)[:-4] + ".o")
        if os.path.exists(obj) and os.path.getmtime(obj) >= max(dep_time, os.path.getmtime(src)):
            return obj
        r = subprocess.run([cxx] + flags + ["-c", src, "-o", obj], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("host emulation build failed:\n" + r.stderr[-4000:])
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, srcs))
    if not os.path.exists(EXE) or os.path.getmtime(EXE) < max(os.path.getmtime(o) for o in objs):
        subprocess.run([cxx] + flags + objs + ["-o", EXE], check=True)
    return EXE


if __name__ == "__main__":
    print(build())
