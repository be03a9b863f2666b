"""Build libntk.so in-tree: nvcc, sm_103a, one -gencode, parallel TUs.

The library is written next to this file (ntk/libntk.so) so the process that
uses it loads it from the source tree.  Sources are compiled to objects in
parallel and linked with nvcc -shared; only stale objects are rebuilt.
"""
import concurrent.futures
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libntk.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + INCLUDE]


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(INCLUDE, "ntk.h"))
    return hs


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths if os.path.exists(p)), default=0.0)


def build(verbose=False, extra_flags=(), out=None, build_dir=None):
    """Compile stale objects and link libntk.so.  out/build_dir/extra_flags
    build a variant elsewhere (used for tuning experiments)."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        raise RuntimeError("nvcc not found; libntk.so cannot be built")
    lib_path = out or LIB
    bdir = build_dir or BUILD
    os.makedirs(bdir, exist_ok=True)
    hdr_time = max(_newest(_headers()), os.path.getmtime(__file__))
    jobs = []
    objs = []
    for src in _sources():
        obj = os.path.join(bdir, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_time):
            jobs.append((src, obj))

    def compile_one(job):
        src, obj = job
        cmd = [nvcc] + NVCC_FLAGS + list(extra_flags) + ["-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if res.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (os.path.basename(src), res.stdout))
        return res.stdout

    logs = []
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            logs = list(ex.map(compile_one, jobs))
    if jobs or not os.path.exists(lib_path) or os.path.getmtime(lib_path) < _newest(objs):
        cmd = [nvcc, ARCH, "-shared", "-o", lib_path] + objs + ["-lcudart"]
        res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed:\n%s" % res.stdout)
    if verbose:
        return lib_path, "\n".join(logs)
    return lib_path


if __name__ == "__main__":
    import sys

    out = build(verbose="-v" in sys.argv)
    print(out if isinstance(out, str) else out[0] + "\n" + out[1])
