"""Time the reference's own GPU pipeline on this GPU (TEST INFRASTRUCTURE).

Runs experiments/run-compact.py:47-90 with the reference's kernels compiled
for this GPU (oracle/ref_gpu.cu over the rendered reference source, built by
oracle/build.py): dfdx = compute_rhs + NearToeplitzSolver.solve; dfdy and dfdz
add the two permutes.  Prints one JSON line with ms per derivative and rows/s,
the reference-kernel baseline for the 512^3 three-direction derivative.

    python oracle/time_reference_gpu.py [N] [reps]
    python oracle/time_reference_gpu.py adi [N] [steps]

The `adi` form times experiments/run-adi.py:59-71 instead (stencil, CR
solve of rows 1..N-2, transpose, twice per step) on an N x N field.
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "near-toeplitz-applications_gb300"))


def main_adi(N, steps):
    import numpy as np
    import torch

    import oracle as O
    from ntk.workloads import gaussians_2d

    R = O.ref_gpu()
    if R is None:
        print(json.dumps({"unavailable": "reference kernels not built (oracle/_ref missing)"}))
        return 0
    dev = torch.device("cuda", 0)
    dx = 1.0 / (N - 1)
    dt = 2 * 0.5 * dx * dx  # r = 0.5
    co = O.adi_coeffs(dx, dt)  # experiments/run-adi.py:50-53
    u = gaussians_2d(N, seed=0, device=dev)
    d_x = u.clone()
    d_y = u.t().contiguous()
    arrs = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in O.precompute(N, co)]
    s = torch.cuda.current_stream().cuda_stream

    def solve(x):  # rows 1..N-2, in place (experiments/run-adi.py:65)
        assert R.ntkref_gpu_cr(N, N - 2, *[a.data_ptr() for a in arrs], co[0], co[1], co[2], co[3], co[4],
                               x.data_ptr() + 8 * N, s) == 0

    def step():
        assert R.ntkref_gpu_adi_rhs(u.data_ptr(), d_x.data_ptr(), N, dx, dt, s) == 0
        solve(d_x)
        assert R.ntkref_gpu_transpose(d_x.data_ptr(), u.data_ptr(), N, s) == 0
        assert R.ntkref_gpu_adi_rhs(u.data_ptr(), d_y.data_ptr(), N, dx, dt, s) == 0
        solve(d_y)
        assert R.ntkref_gpu_transpose(d_y.data_ptr(), u.data_ptr(), N, s) == 0

    for _ in range(3):
        step()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    rows = 2 * (N - 2) * N
    print(json.dumps({"workload": "reference kernels, ADI %d^2, r = 0.5" % N, "ms_per_step": ms,
                      "rows_per_s": rows / (ms * 1e-3)}))
    return 0


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "adi":
        return main_adi(int(sys.argv[2]) if len(sys.argv) > 2 else 2048, int(sys.argv[3]) if len(sys.argv) > 3 else 20)
    import numpy as np
    import torch

    import oracle as O
    from ntk.workloads import fourier_field

    R = O.ref_gpu()
    if R is None:
        print(json.dumps({"unavailable": "reference kernels not built (oracle/_ref missing)"}))
        return 0
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 512
    reps = int(sys.argv[2]) if len(sys.argv) > 2 else 10
    dev = torch.device("cuda", 0)
    co = (1., 2., 1. / 4, 1., 1. / 4, 2., 1.)  # experiments/run-compact.py:48
    h = 1.0 / (n - 1)
    f = fourier_field((n, n, n), seed=0, device=dev)
    tmp = torch.empty_like(f)
    g = torch.empty_like(f)
    out = torch.empty_like(f)
    arrs = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in O.precompute(n, co)]
    s = torch.cuda.current_stream().cuda_stream
    st = [n * n, n, 1]

    def solve(x):
        assert R.ntkref_gpu_cr(n, n * n, *[a.data_ptr() for a in arrs], co[0], co[1], co[2], co[3], co[4],
                               x.data_ptr(), s) == 0

    def perm(a, b, p):
        ss = [st[i] for i in p]
        assert R.ntkref_gpu_permute(a.data_ptr(), b.data_ptr(), n, n, n, ss[0], ss[1], ss[2], s) == 0

    def dfdx():
        assert R.ntkref_gpu_compact_rhs(f.data_ptr(), out.data_ptr(), n, n, n, h, s) == 0
        solve(out)

    def dfdy():
        perm(f, g, (0, 2, 1))
        assert R.ntkref_gpu_compact_rhs(g.data_ptr(), tmp.data_ptr(), n, n, n, h, s) == 0
        solve(tmp)
        perm(tmp, out, (0, 2, 1))

    def dfdz():
        perm(f, g, (1, 2, 0))
        assert R.ntkref_gpu_compact_rhs(g.data_ptr(), tmp.data_ptr(), n, n, n, h, s) == 0
        solve(tmp)
        perm(tmp, out, (2, 0, 1))

    res = {"workload": "reference kernels, compact derivative of a %d^3 field" % n}
    total = 0.0
    for name, fn in (("dfdx", dfdx), ("dfdy", dfdy), ("dfdz", dfdz)):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        res[name + "_ms"] = ms
        total += ms
    res["ms_per_step"] = total
    res["rows_per_s"] = 3 * n ** 3 / (total * 1e-3)
    # and the solve alone (the CR kernel, in place, n^2 systems)
    for _ in range(2):
        solve(out)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        solve(out)
    e1.record()
    torch.cuda.synchronize()
    res["cr_solve_ms"] = e0.elapsed_time(e1) / reps
    print(json.dumps(res))
    return 0


if __name__ == "__main__":
    sys.exit(main())
