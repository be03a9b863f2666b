"""Render the reference's CUDA kernel templates into oracle/_ref/.

TEST INFRASTRUCTURE ONLY (part of the parity checker, never the product).

The reference (ashwinsrnth/near-toeplitz-applications) keeps every GPU kernel
as CUDA C in a Python string, some of them jinja2 templates, and compiles
them at run time with PyCUDA.  This script reads those strings out of the
reference's source files with `ast` (the Python 2 modules are never imported
or executed), renders them exactly as the reference does, and writes them to
oracle/_ref/ref_kernels.cuh, each kernel in its own C++ namespace:

  neato.py:7-125, rendered as neato.py:160-161 for n = 4 ... 2048
                              -> namespace ntkref_cr_n<n>
  compact/rhs.py:8-38         -> namespace ntkref_rhs
  compact/permute.py:6-21     -> namespace ntkref_permute
  adi/rhs.py:10-25            -> namespace ntkref_adi_rhs
  adi/transpose.py:9-27, rendered with TILE_DIM = BLOCK_ROWS = 32
                              (adi/transpose.py:47)
                              -> namespace ntkref_transpose

oracle/ref_cpu.cpp (g++, CPU emulation of the CUDA execution model) and
oracle/ref_gpu.cu (nvcc) include that header.  oracle/_ref/ is git-ignored:
the rendered reference source is never committed.

Usage: python oracle/render_ref.py [REFERENCE_ROOT]
Exits 0 without writing anything when the reference tree is absent.
"""
import ast
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
OUT = os.path.join(OUT_DIR, "ref_kernels.cuh")
CR_SIZES = [4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048]


def _string_constant(path, name):
    with open(path, "r") as fh:
        tree = ast.parse(fh.read(), filename=path)
    for node in tree.body:
        if isinstance(node, ast.Assign) and len(node.targets) == 1:
            tgt = node.targets[0]
            if isinstance(tgt, ast.Name) and tgt.id == name and isinstance(node.value, ast.Constant):
                return node.value.value
    raise KeyError("%s not found in %s" % (name, path))


def render(ref_root):
    import jinja2  # only needed where the reference tree exists

    parts = ["// Generated by oracle/render_ref.py from the reference sources. Do not commit.\n",
             "#pragma once\n"]
    cr = jinja2.Template(_string_constant(os.path.join(ref_root, "neato.py"), "kernel_template"))
    for n in CR_SIZES:
        # neato.py:160-161: tpl.render(n=self.n, shared_size=self.n/2)
        parts.append("namespace ntkref_cr_n%d {\n%s\n}\n" % (n, cr.render(n=n, shared_size=n / 2)))
    parts.append("namespace ntkref_rhs {\n%s\n}\n"
                 % _string_constant(os.path.join(ref_root, "compact", "rhs.py"), "kernel_template"))
    parts.append("namespace ntkref_permute {\n%s\n}\n"
                 % _string_constant(os.path.join(ref_root, "compact", "permute.py"), "kernel_text"))
    parts.append("namespace ntkref_adi_rhs {\n%s\n}\n"
                 % _string_constant(os.path.join(ref_root, "adi", "rhs.py"), "kernel_template"))
    tr = jinja2.Template(_string_constant(os.path.join(ref_root, "adi", "transpose.py"), "kernel_template"))
    parts.append("namespace ntkref_transpose {\n%s\n}\n" % tr.render(TILE_DIM=32, BLOCK_ROWS=32))
    parts.append("#define NTKREF_CR_SIZES(X) %s\n" % " ".join("X(%d)" % n for n in CR_SIZES))
    os.makedirs(OUT_DIR, exist_ok=True)
    text = "".join(parts)
    old = open(OUT).read() if os.path.exists(OUT) else None
    if old != text:
        with open(OUT, "w") as fh:
            fh.write(text)
    return OUT


def precompute_coefficients_from_reference(ref_root):
    """Return the reference's own _precompute_coefficients (neato.py:199-274).

    The function's source is taken out of neato.py with `ast` and executed on
    its own (the module's pycuda imports are skipped).  Its body is valid
    Python 3 and uses only numpy."""
    import numpy as np

    path = os.path.join(ref_root, "neato.py")
    with open(path) as fh:
        src = fh.read()
    tree = ast.parse(src)
    fn = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == "_precompute_coefficients"][0]
    mod = ast.Module(body=[fn], type_ignores=[])
    ns = {"np": np}
    exec(compile(mod, path, "exec"), ns)
    return ns["_precompute_coefficients"]


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("NTK_REFERENCE_ROOT", "")
    if not root:
        print("usage: render_ref.py REFERENCE_ROOT (or set NTK_REFERENCE_ROOT)")
        sys.exit(2)
    if not os.path.isfile(os.path.join(root, "neato.py")):
        print("reference tree not found at %s; nothing rendered" % root)
        sys.exit(0)
    print(render(root))
