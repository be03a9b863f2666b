"""Build recipe for the parity checker (TEST INFRASTRUCTURE ONLY).

  oracle/libntk_oracle.so      gcc   ntk_oracle.c (CPU restatement of the reference)
  oracle/_ref/libntkref_cpu.so g++   ref_cpu.cpp + the rendered reference kernels,
                                     executed on the CPU
  oracle/_ref/libntkref_gpu.so nvcc  ref_gpu.cu + the rendered reference kernels,
                                     compiled for sm_103a

The rendered kernels (oracle/_ref/ref_kernels.cuh) are produced by
oracle/render_ref.py where the reference tree exists; elsewhere the two
oracle/_ref libraries are built only if that header is already present.
Every library is rebuilt only when a source is newer than it.
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
REF_HDR = os.path.join(REF_DIR, "ref_kernels.cuh")
ORACLE_SO = os.path.join(HERE, "libntk_oracle.so")
REF_CPU_SO = os.path.join(REF_DIR, "libntkref_cpu.so")
REF_GPU_SO = os.path.join(REF_DIR, "libntkref_gpu.so")
# Root of the reference's source tree: given to build_all() or taken from
# NTK_REFERENCE_ROOT; with neither, or where the tree is absent, only the
# oracle and an already rendered oracle/_ref header are built.
REFERENCE_ROOT = os.environ.get("NTK_REFERENCE_ROOT")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources if os.path.exists(s))


def _run(cmd, cwd=HERE):
    res = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), res.stdout))


def build_oracle():
    src = os.path.join(HERE, "ntk_oracle.c")
    if _stale(ORACLE_SO, [src, __file__]):
        _run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", ORACLE_SO, src, "-lm"])
    return ORACLE_SO


def render_reference():
    """Render the reference kernels when the reference tree is present."""
    if REFERENCE_ROOT and os.path.isfile(os.path.join(REFERENCE_ROOT, "neato.py")):
        from importlib import util

        spec = util.spec_from_file_location("_ntk_render_ref", os.path.join(HERE, "render_ref.py"))
        mod = util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.render(REFERENCE_ROOT)
    return os.path.exists(REF_HDR)


def build_ref_cpu():
    if not render_reference():
        return None
    src = os.path.join(HERE, "ref_cpu.cpp")
    if _stale(REF_CPU_SO, [src, REF_HDR, __file__]):
        _run(["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-o", REF_CPU_SO, src])
    return REF_CPU_SO


def build_ref_gpu():
    if not render_reference() or shutil.which("nvcc") is None:
        return None
    src = os.path.join(HERE, "ref_gpu.cu")
    if _stale(REF_GPU_SO, [src, REF_HDR, __file__]):
        _run(["nvcc", ARCH, "-O2", "-lineinfo", "-Xcompiler", "-fPIC", "-shared", "-o", REF_GPU_SO, src])
    return REF_GPU_SO


def build_all(reference_root=None):
    """Builds the oracle and, when the reference tree is at reference_root
    (or NTK_REFERENCE_ROOT), the rendered reference kernels."""
    global REFERENCE_ROOT
    if reference_root:
        REFERENCE_ROOT = reference_root
    out = {"oracle": build_oracle()}
    try:
        out["ref_cpu"] = build_ref_cpu()
    except RuntimeError as exc:  # the checker must not block the product build
        out["ref_cpu"] = None
        out["ref_cpu_error"] = str(exc)[:400]
    try:
        out["ref_gpu"] = build_ref_gpu()
    except RuntimeError as exc:
        out["ref_gpu"] = None
        out["ref_gpu_error"] = str(exc)[:400]
    return out


if __name__ == "__main__":
    import sys

    print(build_all(sys.argv[1] if len(sys.argv) > 1 else None))
