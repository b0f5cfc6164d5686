"""One named factorization on device data, run a few times: the target of
profiler captures (ncu -k <kernel> -c <launches> python -m zml_gb300.cases ...).

    python -m zml_gb300.cases dgetrf 4096 [--reps 2] [--fp64-updates 1]

Cases (seeded N(0,1) inputs; SPD inputs G G^T / n + I):
  dgetrf, dpotrf        FP64 LU / Cholesky (zml_gpu_dgetrf, zml_gpu_dpotrf)
  dgemm_slices          C (n x n) -= A (n x 256) B (256 x n) in FP64 by the exact-slice
                        GEMM (the LU's trailing update)
  mixed                 n x n Ax=b, BF16x3 LU + GMRES-IR (zml_gpu_dgesv_mpir)
  zgeqrf, dsytrf        complex QR, Bunch-Kaufman (device pointers, C entries)
Each run is timed with CUDA events and printed with its return code.
"""
import argparse
import ctypes as C

from . import MpirResult, last_error, lib, profile_read


def main():
    import torch
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("case", choices=["dgetrf", "dpotrf", "dgemm_slices", "mixed", "zgeqrf",
                                     "dsytrf"])
    ap.add_argument("n", type=int)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--profile", action="store_true",
                    help="one more run with per-launch CUDA events: time per kernel class")
    ap.add_argument("--fp64-updates", type=int, default=1,
                    help="1: FP64 trailing updates by exact slices on the tensor cores "
                         "(above the size threshold), 0: on the FP64 pipe")
    a = ap.parse_args()
    L = lib()
    L.zml_gpu_fp64_updates(a.fp64_updates)
    n = a.n
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev).manual_seed(5)
    st = torch.cuda.current_stream().cuda_stream
    info = C.c_int(0)
    S = torch.randn(n, n, dtype=torch.float64, device=dev, generator=g)
    if a.case == "dpotrf":
        S = S @ S.t() / n + torch.eye(n, dtype=torch.float64, device=dev)
    piv = torch.zeros(n, dtype=torch.int32, device=dev)
    F = S.clone()
    b = torch.rand(n, 1, dtype=torch.float64, device=dev, generator=g) * 2 - 1
    x = torch.zeros_like(b)
    res = MpirResult()
    if a.case == "zgeqrf":
        Z = torch.randn(n, n, dtype=torch.complex128, device=dev, generator=g)
        ZF = Z.clone()
        tau = torch.zeros(n, dtype=torch.complex128, device=dev)
    if a.case == "dsytrf":
        S = (S + S.t()) / 2
    if a.case == "dgemm_slices":
        B2 = torch.randn(n, 256, dtype=torch.float64, device=dev, generator=g)  # storage of B^T
        C2 = torch.zeros(n, n, dtype=torch.float64, device=dev)

    def run():
        if a.case == "dgetrf":
            F.copy_(S)
            return L.zml_gpu_dgetrf(n, n, F.data_ptr(), n, piv.data_ptr(), C.byref(info), st)
        if a.case == "dpotrf":
            F.copy_(S)
            return L.zml_gpu_dpotrf(b"L", n, F.data_ptr(), n, C.byref(info), st)
        if a.case == "dgemm_slices":
            return L.zml_gpu_dgemm_slices(n, n, 256, S.data_ptr(), n, B2.data_ptr(), 256,
                                          C2.data_ptr(), n, 0, st)
        if a.case == "mixed":
            return L.zml_gpu_dgesv_mpir(n, 1, S.data_ptr(), n, b.data_ptr(), n, x.data_ptr(), n,
                                        3, 1, 64 * 2.0 ** -53, 30, C.byref(res), st)
        if a.case == "zgeqrf":
            ZF.copy_(Z)
            return L.LAPACKE_zgeqrf(102, n, n, ZF.data_ptr(), n, tau.data_ptr())
        F.copy_(S)
        return L.LAPACKE_dsytrf(102, b"L", n, F.data_ptr(), n, piv.data_ptr())

    for r in range(a.reps):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rc = run()
        e1.record()
        torch.cuda.synchronize()
        print("%s n=%d rep %d: rc %d, %.3f ms%s" % (a.case, n, r, rc, e0.elapsed_time(e1),
                                                     "" if rc == 0 else " " + last_error()))
        if rc != 0:
            raise SystemExit(1)
    if a.profile:
        L.zml_gpu_profile(1)
        run()
        torch.cuda.synchronize()
        prof = profile_read()
        L.zml_gpu_profile(0)
        for name, (cnt, ms, fl, by) in sorted(prof.items(), key=lambda kv: -kv[1][1]):
            print("  %-10s %6d launches %9.3f ms %8.2f TFLOP/s %8.1f GB/s"
                  % (name, cnt, ms, fl / ms / 1e9 if ms else 0, by / ms / 1e6 if ms else 0))


if __name__ == "__main__":
    main()
