"""In-tree build of the CUDA library ``astrea_gb300/_lib/libastrea_gb300.so``.

Every translation unit is compiled by its own ``nvcc`` process (in parallel)
for sm_103a only, then linked with ``nvcc -shared``.  FP64 sweep units and the
API unit are compiled without fused multiply-add (``--fmad=false``) so the
plain FP64 path rounds exactly like the reference's NumPy expressions; the
FP32 sweep units keep FMA.

Usage: ``python -m astrea_gb300.build [-j N] [--force]``
"""

import argparse
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libastrea_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-diag-suppress", "177"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def flags_for(name):
    if name.startswith(("sweep_f32", "batch_k_f32", "cellavg_f32")):
        # FP32 path: fused multiply-add, approximate division and square root, flush-to-zero
        return ["--fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]
    return ["--fmad=false"]


def _digest(paths, extra):
    h = hashlib.sha256()
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(" ".join(extra).encode())
    return h.hexdigest()[:16]


def build(jobs=None, force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h")))
    headers.append(os.path.join(HERE, "..", "include", "astrea_gb300.h"))
    nv = nvcc()
    cmds = []
    objs = []
    for src in sources():
        cu = os.path.join(CSRC, src)
        fl = COMMON + ARCH + flags_for(src)
        key = _digest([cu] + headers, fl)
        obj = os.path.join(BUILD_DIR, f"{src[:-3]}.{key}.o")
        objs.append(obj)
        if force or not os.path.exists(obj):
            cmds.append((src, [nv] + fl + ["-c", cu, "-o", obj]))
    # longest units first (batched kernels, then the high-order sweeps) so the pool drains evenly
    cmds.sort(key=lambda c: (not c[0].startswith("batch_k"), not c[0].startswith(("sweep_f64", "sweep_f32_w")), c[0]))
    jobs = jobs or max(1, min(len(cmds), os.cpu_count() or 4))
    if cmds:
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            futs = {ex.submit(subprocess.run, c, capture_output=True, text=True): s for s, c in cmds}
            for fut in cf.as_completed(futs):
                r = fut.result()
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed on {futs[fut]}:\n{r.stderr[-4000:]}")
                if verbose:
                    print(f"compiled {futs[fut]}", flush=True)
    link_key = _digest(objs, [])
    stamp = LIB + ".stamp"
    if force or not os.path.exists(LIB) or not os.path.exists(stamp) or open(stamp).read() != link_key:
        tmp = LIB + ".tmp"
        r = subprocess.run([nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
        os.replace(tmp, LIB)
        with open(stamp, "w") as f:
            f.write(link_key)
    # drop stale objects of earlier source versions
    keep = set(objs)
    for f in os.listdir(BUILD_DIR):
        p = os.path.join(BUILD_DIR, f)
        if p.endswith(".o") and p not in keep:
            os.remove(p)
    return LIB


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("-j", type=int, default=None)
    ap.add_argument("--force", action="store_true")
    args = ap.parse_args(argv)
    print(build(args.j, args.force, verbose=True))


if __name__ == "__main__":
    sys.exit(main())
