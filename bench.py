"""Benchmark: batched angular power spectra on GB300.

Workload (the batched configuration of the benchmark set): 4096 cosmologies
drawn from a seeded uniform box (Omega_c in [0.20, 0.35], Omega_b in
[0.04, 0.06], h in [0.60, 0.80], n_s in [0.90, 1.00], sigma8 in [0.60, 1.00],
w0 in [-1.3, -0.7], wa = 0, Omega_k = 0), 5 WeakLensing smail_nz bins (a = 1,
b = 2, z0 = linspace(0.3, 1.5, 5), zmax = 10), 100 log-spaced ell in
[20, 3000], Limber N = 512.  15 spectra per cosmology, 6.144M C_ell per step.

A step is one angular_cl pass over the whole batch: background tables, halofit
rows, tracer kernels, Limber integral (fp32c: float32 integrand with
compensated sums, float64 tables).  ``value`` is C_ell evaluations per second
with inputs resident in HBM; ``e2e`` is the same through the public API with
the parameters copied from pinned host memory and the C_ell copied back each
step.  The plain float64 method is timed on the same workload as
``fp64_value``.

Beside the headline: the plain float64 method one cosmology per call (the
per-cosmology rate the batched form is compared with), C_ell plus the Jacobian
dC_ell/dtheta over the whole batch (``cl_grad``), and the serving loop under 64
synthetic HMC chains (``serving``: requests/s, p50/p99 log-likelihood+gradient
latency).

``--impl reference`` times the CPU reference of the path instead (the float64
oracle port on the host cores; JAX is not available on the GPU host).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

B_DEFAULT = 4096
N_ELL = 100
Z0 = np.linspace(0.3, 1.5, 5)
SEED = 20261203
BOX = {
    "Omega_c": (0.20, 0.35),
    "Omega_b": (0.04, 0.06),
    "h": (0.60, 0.80),
    "n_s": (0.90, 1.00),
    "sigma8": (0.60, 1.00),
    "w0": (-1.3, -0.7),
}
ORDER = ["Omega_c", "Omega_b", "h", "n_s", "sigma8", "Omega_k", "w0", "wa"]
# Per-cosmology figures of the fp32c step's kernels on this workload (na = 513
# Limber nodes, 5 WL tracers, 100 ell), from ncu captures at 2048 cosmologies
# (working sets above L2; the table stage's traffic at 4096), one kernel per
# capture (profiles/fp32c_kernels_b2048_per_kernel.md), per cosmology:
#   warp instructions issued (sm__inst_executed); the table stage is
#     cosmo_scalars_kernel + cosmo_tables_kernel;
#   FP64 operations = DFMA x 2 + DADD + DMUL thread instructions;
#   traffic = dram__bytes_read.sum + dram__bytes_write.sum;
#   per Limber node (100 x 513 per cosmology): XU (MUFU) thread operations
#     and warp instructions of limber32_kernel.
WARP_INSTR_PER_COSMO = {"cosmo_tables": 1_984 + 79_846, "halofit_rows": 95_982, "tracer_kernels": 123_066}
FP64_OPS = {"cosmo_tables": 14_262 + 26_309, "halofit_rows": 28_728}
TRAFFIC_PER_COSMO = {"cosmo_tables": 79 + 42_725, "halofit_rows": 160_853, "tracer_kernels": 4_150, "limber": 51_366}
# the table stage writes its 55,104-byte record and reads little: its traffic
# is taken at the benched batch (4096), and what the L2 still holds of its
# writes when the kernel ends reaches DRAM after it
TRAFFIC_NOTE = {"cosmo_tables": "DRAM bytes of the kernels at 4096 cosmologies; up to one L2 (126 MB) of the "
                                "226 MB of records they write is written back after the kernel ends"}
MUFU_PER_NODE = 17.36
WARP_INSTR_PER_NODE = 8.109
# algorithmic bytes per cosmology: what each kernel must read and write once
#   cosmo_tables: 8 parameters in, the CosmoTab record out (55,104 B)
#   halofit_rows: the CosmoTab record in, FP64 + FP32 rows and the float
#     Limber weight out (513 x (7 x 8 + 16 x 4 + 4))
#   tracer_kernels: the FP32 chi table and slopes in (2 x 256 x 4), 5 float kernels out (5 x 513 x 4)
#   limber: FP32 rows (16 x 4) + u (4) + 5 float radial kernels (5 x 4) per node in, 15 x 100 C_ell out
ALG_BYTES = {"cosmo_tables": 64 + 55_104, "halofit_rows": 55_104 + 513 * (7 * 8 + 16 * 4 + 4),
             "tracer_kernels": 2 * 256 * 4 + 5 * 513 * 4,
             "limber": 513 * (16 * 4 + 4) + 5 * 513 * 4 + 15 * N_ELL * 8}
# the fp32c vector-Jacobian product's stages (jcg_calib_vjp_stages masks) and
# their per-cosmology figures from the same captures: warp instructions,
# traffic, and algorithmic bytes (inputs read once, outputs written once,
# scratch excluded):
#   tables: parameters in; the TabD record (122,944 B) and the Taylor tables
#     (206,592 B) out.  Kernels: grad_scalars32, grad_nodes<0..2>, grad_tables,
#     grad_moments32;
#   rows: TabD's float copies, P(k) and Taylor tables in (245,152 B), rows
#     out (513 x 132 x 4);
#   kernels: the chi table in (2 x 256 x 4), the values of 5 radial kernels
#     out (5 x 513 x 4; their zero tangents are not stored).  grad_kernval32u
#     (its traffic is above these bytes: each 4-byte value lands in a 36-byte
#     record, so the L2 reads the sector before merging it);
#   product: rows, radial kernels, cotangent and Eisenstein-Hu inputs in;
#     C_ell, the shear kernels' cotangents and the chunk gradients out.
#     grad_vjp32 (the dominant kernel: 22.25 warp instructions and 35.5 MUFU
#     operations per Limber node);
#   reverse: the shear cotangents and the chi table's tangents in, the chunk
#     gradients out.  kernrev_owner, grad_kernrev32u, vjp_grad_reduce.
VJP_STAGES = (("tables", 1), ("rows", 2), ("kernels", 4), ("product", 8), ("reverse", 16))
VJP_WARP_INSTR_PER_COSMO = {"tables": 338 + 9_420 + 5_970 + 39_574 + 22_665 + 69_596, "rows": 126_589,
                            "kernels": 122_006, "product": 1_141_466, "reverse": 211 + 280_478 + 112}
VJP_TRAFFIC_PER_COSMO = {"tables": 346 + 3_339 + 3_320 + 3_077 + 104_278 + 218_538, "rows": 485_339,
                         "kernels": 157_559, "product": 397_623, "reverse": 261 + 21_404 + 3_206}
VJP_ALG_BYTES = {"tables": 64 + 122_944 + 206_592, "rows": 245_152 + 513 * 132 * 4,
                 "kernels": 2 * 256 * 4 + 5 * 513 * 4,
                 "product": 513 * 132 * 4 + 5 * 513 * 9 * 4 + 15 * N_ELL * 8 + 416 + 15 * N_ELL * 8 + 5 * 513 * 4
                 + 17 * 8 * 8,
                 "reverse": 5 * 513 * 4 + 2 * 8 * 256 * 4 + 33 * 8 * 8}
VJP_PRODUCT_WARP_INSTR_PER_NODE = 22.25
VJP_PRODUCT_MUFU_PER_NODE = 35.5
KERNEL_NAMES = {"cosmo_tables": "cosmo_scalars_kernel + cosmo_tables_kernel",
                "halofit_rows": "halofit_rows_kernel<fp32c>",
                "tracer_kernels": "tracer32_uniform_kernel<5>", "limber": "limber32_kernel<1>"}


def draw_params(B, seed=SEED):
    rng = np.random.default_rng(seed)
    P = np.zeros((B, 8))
    for i, n in enumerate(ORDER):
        if n in BOX:
            lo, hi = BOX[n]
            P[:, i] = rng.uniform(lo, hi, B)
    return P


def ell_grid():
    return np.logspace(np.log10(20.0), np.log10(3000.0), N_ELL)


# ------------------------------------------------------------ CPU baseline --
def _oracle_worker(rows):
    import torch

    torch.set_num_threads(1)
    from oracle import jc_oracle as O

    probes = [O.Probe("wl", [O.Smail(1.0, 2.0, float(z0), 10.0, 10.0) for z0 in Z0], sigma_e=0.26)]
    ell = ell_grid()
    for r in rows:
        O.angular_cl(O.Cosmo.from_vector(r), ell, probes, n_limber=512)
    return len(rows)


def cpu_baseline(params, budget_s=12.0, procs=None):
    """Oracle port on the host cores, spawn pool, bounded to ~budget_s."""
    import multiprocessing as mp

    procs = procs or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    n_cls = 15
    with ctx.Pool(procs) as pool:
        # warm-up: imports and first call in every worker
        pool.map(_oracle_worker, [[params[i % len(params)]] for i in range(procs)])
        done, t0, k = 0, time.perf_counter(), 0
        while time.perf_counter() - t0 < budget_s:
            chunk = [[params[(k + i) % len(params)]] for i in range(procs)]
            k += procs
            done += sum(pool.map(_oracle_worker, chunk))
        dt = time.perf_counter() - t0
    return {
        "value": done * n_cls * N_ELL / dt,
        "unit": "C_ell/s",
        "cores": procs,
        "kind": "port",
        "sample": f"{done} cosmologies of the workload (float64 oracle, one process per core), {dt:.1f} s",
    }


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.skip = 0
        self.path = os.path.join(tempfile.gettempdir(), f"jcg_clocks_{os.getpid()}.csv")

    def _lines(self):
        try:
            with open(self.path) as f:
                return [ln for ln in f.read().split("\n") if ln.count(",") >= 8]
        except OSError:
            return []

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "10"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # the sampler is running once its first line is out; samples before
        # mark() (idle) are not counted
        t0 = time.time()
        while not self._lines() and time.time() - t0 < 5.0 and self.proc.poll() is None:
            time.sleep(0.01)

    def mark(self):
        self.skip = len(self._lines())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        lines = self._lines()
        for line in (lines[self.skip:] or lines[-1:]):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                                "sw_power_cap"], f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------- GPU arm ----
def gpu_arm(args, rank, world, device):
    import torch

    import jax_cosmo_gb300 as jc
    from jax_cosmo_gb300 import _geometry, _lib
    from jax_cosmo_gb300.angular_cl import angular_cl_device

    B = args.batch
    P = draw_params(B, SEED + rank)
    nz = [jc.redshift.smail_nz(1.0, 2.0, float(z0), gals_per_arcmin2=10.0) for z0 in Z0]
    probes = [jc.probes.WeakLensing(nz, sigma_e=0.26)]
    ell_np = ell_grid()
    params = torch.as_tensor(P, device=device).contiguous()
    n_cls, n_ell = 15, N_ELL
    cl = torch.empty(B, n_cls, n_ell, dtype=torch.float64, device=device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)  # > L2 (126 MB)
    stream = torch.cuda.current_stream(device)

    def step(prec):
        angular_cl_device(params, ell_np, probes, prec, 512, out=cl)

    def timed(fn, K, W):
        for _ in range(W):
            fn()
        torch.cuda.synchronize(device)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(device)
        times = []
        for _ in range(K):
            flush.fill_(1.0)  # evict L2 between timed iterations (not timed)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        torch.cuda.synchronize(device)
        return float(np.sum(times)), times

    if args.fwd_only:
        # the fp32c angular_cl step alone (a profiling entry)
        tf, _ = timed(lambda: step("fp32c"), args.steps, args.warmup)
        return {"jacobian_only": {"batch": B, "ms_per_step": tf / args.steps, "what": "C_ell fp32c",
                                  "cl_per_s": B * 15 * N_ELL / (tf / args.steps * 1e-3)}}
    if args.vjp_only:
        # the fp32c C_ell + vector-Jacobian product alone (a profiling entry)
        from jax_cosmo_gb300.autodiff import vjp_device

        gen = torch.Generator(device=device).manual_seed(SEED)
        vb = torch.randn(B, 15, N_ELL, generator=gen, dtype=torch.float64, device=device)
        tv, _ = timed(lambda: vjp_device(params, ell_np, probes, vb, 512, "fp32c", want_cl=True), args.steps,
                      args.warmup)
        return {"jacobian_only": {"batch": B, "ms_per_step": tv / args.steps, "what": "C_ell + VJP",
                                  "cl_grad_per_s": B * 15 * N_ELL / (tv / args.steps * 1e-3)}}
    if args.jacobian_only:
        # the fp32c Jacobian alone (a profiling entry: one kernel family per launch list)
        from jax_cosmo_gb300.autodiff import jacobian_device

        tj, _ = timed(lambda: jacobian_device(params, ell_np, probes, 512, "fp32c"), args.steps, args.warmup)
        return {"jacobian_only": {"batch": B, "ms_per_step": tj / args.steps,
                                  "cl_grad_per_s": B * 15 * N_ELL / (tj / args.steps * 1e-3)}}

    # headline: fp32c, inputs resident
    clocks = ClockSampler(device.index)
    clocks.start()
    clocks.mark()
    t_fast, per = timed(lambda: step("fp32c"), args.steps, args.warmup)
    clk = clocks.stop()
    # plain float64 method on the same workload (fewer steps: it is ~100x slower)
    t64, per64 = timed(lambda: step("fp64"), max(1, min(args.steps, 2)), 1)
    # e2e through the public host-buffer entry (jcg_angular_cl_host): pinned
    # host params in, C_ell out to pinned host memory, both inside each step
    host_p = torch.as_tensor(P).pin_memory()
    host_cl = torch.empty(B, n_cls, n_ell, dtype=torch.float64).pin_memory()

    def e2e_step():
        jc.cl.angular_cl_host(host_p, ell_np, probes, precision="fp32c", out=host_cl)

    t_e2e, _ = timed(e2e_step, args.steps, args.warmup)
    # Limber kernel alone (the dominant kernel) for the roofline, same stream
    g, geo, _ = _geometry.get_geometry(probes, ell_np, 512, device)
    import ctypes

    wsz = ctypes.c_size_t()
    _lib.call("jcg_workspace_size", ctypes.byref(g), B, _lib.FP32C, ctypes.byref(wsz))
    ws = _lib.workspace(wsz.value, device)
    st = _lib.stream_of(device)
    args_common = (ctypes.byref(g), _lib.ptr(geo), _lib.ptr(params), B, _lib.FP32C)
    _lib.call("jcg_stage_cosmo_tables", ctypes.byref(g), _lib.ptr(params), B, _lib.FP32C,
              _lib.ptr(ws), ctypes.c_size_t(ws.numel()), st)
    _lib.call("jcg_stage_halofit_rows", *args_common, _lib.ptr(ws), ctypes.c_size_t(ws.numel()), st)
    _lib.call("jcg_stage_tracer_kernels", *args_common, _lib.ptr(ws), ctypes.c_size_t(ws.numel()), st)
    t_limber, per_l = timed(
        lambda: _lib.call("jcg_stage_limber", *args_common, _lib.ptr(cl), _lib.ptr(ws),
                          ctypes.c_size_t(ws.numel()), st), args.steps, args.warmup)
    ms_limber = t_limber / args.steps
    stages = {}
    for name in ("jcg_stage_cosmo_tables", "jcg_stage_halofit_rows", "jcg_stage_tracer_kernels"):
        if name == "jcg_stage_cosmo_tables":
            fn = lambda: _lib.call(name, ctypes.byref(g), _lib.ptr(params), B, _lib.FP32C,
                                   _lib.ptr(ws), ctypes.c_size_t(ws.numel()), st)
        else:
            fn = lambda n=name: _lib.call(n, *args_common, _lib.ptr(ws), ctypes.c_size_t(ws.numel()), st)
        t, _ = timed(fn, args.steps, 1)
        stages[name.replace("jcg_stage_", "")] = t / args.steps
    stages["limber"] = ms_limber

    # max over ranks
    def allmax(x):
        if world == 1:
            return x
        tt = torch.tensor([x], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        return float(tt.item())

    t_fast, t64, t_e2e = allmax(t_fast), allmax(t64), allmax(t_e2e)
    ncl_step = B * n_cls * n_ell
    K = args.steps
    res = {
        "t_fast": t_fast, "t64": t64, "n64": len(per64), "t_e2e": t_e2e, "K": K,
        "ncl_step": ncl_step, "clocks": clk, "stages_ms": stages, "ms_limber": ms_limber,
        "h2d": int(host_p.numel() * 8), "d2h": int(host_cl.numel() * 8),
        "sm_count": torch.cuda.get_device_properties(device).multi_processor_count,
    }
    # sanity: the fp32c result vs fp64 on this workload
    step("fp64")
    c64 = cl.clone()
    step("fp32c")
    res["fp32c_max_rel_err_vs_fp64"] = float(((cl - c64).abs() / c64.abs()).max())

    # plain float64 method, one cosmology per call (the per-cosmology rate)
    p1 = params[:1].contiguous()
    cl1 = torch.empty(1, n_cls, n_ell, dtype=torch.float64, device=device)
    t1, _ = timed(lambda: angular_cl_device(p1, ell_np, probes, "fp64", 512, out=cl1), args.steps, args.warmup)
    res["plain_fp64_single"] = {"ms_per_call": t1 / args.steps,
                                "cl_per_s": n_cls * n_ell / (t1 / args.steps * 1e-3)}

    # C_ell + dC_ell/dtheta (8 leaves), whole batch: fp32c and the plain fp64 form
    from jax_cosmo_gb300.autodiff import jacobian_device

    res["jacobian"] = {}
    for prec in ("fp32c", "fp64"):
        kj = max(1, min(args.steps, 5 if prec == "fp32c" else 2))
        tj, _ = timed(lambda p=prec: jacobian_device(params, ell_np, probes, 512, p), kj, 1)
        res["jacobian"][prec] = {"batch": B, "ms_per_step": tj / kj, "steps": kj,
                                 "cl_grad_per_s": ncl_step / (tj / kj * 1e-3)}
    # accuracy of the fp32c Jacobian against the fp64 one (64 cosmologies of the batch)
    p64 = params[:64].contiguous()
    c64, j64 = jacobian_device(p64, ell_np, probes, 512, "fp64")
    c32, j32 = jacobian_device(p64, ell_np, probes, 512, "fp32c")
    scale = j64.abs().amax(dim=(1, 2), keepdim=True)
    res["jacobian"]["fp32c"]["cl_max_rel_err_vs_fp64"] = float(((c32 - c64) / c64).abs().max())
    res["jacobian"]["fp32c"]["jac_max_err_vs_fp64"] = float(((j32 - j64).abs() / scale).max())
    res["jacobian"]["fp32c"]["jac_err_note"] = "max |J32 - J64| / max |J64| per (cosmology, parameter)"
    # C_ell + the gradient of a scalar function of C_ell (a likelihood's
    # backward pass): the vector-Jacobian product, fp32c, with a seeded cotangent
    from jax_cosmo_gb300.autodiff import vjp_device

    gen = torch.Generator(device=device).manual_seed(SEED)
    vb = torch.randn(B, n_cls, n_ell, generator=gen, dtype=torch.float64, device=device)
    kv = max(1, min(args.steps, 5))
    tv, _ = timed(lambda: vjp_device(params, ell_np, probes, vb, 512, "fp32c", want_cl=True), kv, 1)
    g32, c32v = vjp_device(p64, ell_np, probes, vb[:64], 512, "fp32c", want_cl=True)
    gref = torch.einsum("bpl,bpld->bd", vb[:64], j64)
    gscale = torch.einsum("bpl,bpld->bd", vb[:64].abs(), j64.abs())
    # each stage of the fp32c product alone (jcg_calib_vjp_stages on a workspace
    # a full call filled), for the per-kernel rooflines
    import ctypes

    gv_, geov_, _ = _geometry.get_geometry(probes, ell_np, 512, device, 0)
    wszv = ctypes.c_size_t()
    _lib.call("jcg_vjp_workspace_size", ctypes.byref(gv_), B, _lib.FP32C, ctypes.byref(wszv))
    wsv = _lib.workspace(wszv.value, device)
    grad_v = torch.empty(B, 8, dtype=torch.float64, device=device)
    cl_v = torch.empty(B, n_cls, n_ell, dtype=torch.float64, device=device)
    stv = _lib.stream_of(device)

    def vstage(mask):
        _lib.call("jcg_calib_vjp_stages", ctypes.byref(gv_), _lib.ptr(geov_), _lib.ptr(params), B, _lib.ptr(vb),
                  _lib.ptr(cl_v), _lib.ptr(grad_v), _lib.ptr(wsv), ctypes.c_size_t(wsv.numel()), ctypes.c_uint(mask),
                  stv)

    vstage(31)
    vjp_stages = {}
    for name, mask in VJP_STAGES:
        t, _ = timed(lambda m=mask: vstage(m), kv, 1)
        vjp_stages[name] = t / kv
    del wsv
    res["jacobian"]["fp32c_vjp"] = {
        "batch": B, "ms_per_step": tv / kv, "steps": kv, "cl_grad_per_s": ncl_step / (tv / kv * 1e-3),
        "stages_ms": vjp_stages, "rooflines": vjp_rooflines(vjp_stages, B, {"sm_count": torch.cuda.get_device_properties(device).multi_processor_count, "clocks": clk}),
        "what": "C_ell and the gradient of a scalar of C_ell (vector-Jacobian product with a seeded cotangent; "
                "the Jacobian is not formed)",
        "grad_max_err_vs_fp64": float(((g32 - gref).abs() / gscale).max()),
        "cl_max_rel_err_vs_fp64": float(((c32v - c64) / c64).abs().max()),
        "err_note": "max |g32 - J64^T v| / (|v|^T |J64|) per (cosmology, parameter)"}
    del j64, j32

    # the non-default operator points on the same workload (fp32c), each with
    # its error against the plain fp64 method of the same operator points
    params_g = torch.cat([params, torch.full((B, 1), 0.55, dtype=torch.float64, device=device)], dim=1)
    c64v = torch.empty_like(cl)
    res["operator_points"] = {}
    for name, phys in (("halofit_smith2003", _lib.PK_SMITH2003), ("linear_matter_power", _lib.PK_LINEAR),
                       ("eisenhu_nowiggle", _lib.TF_NOWIGGLE), ("gamma_growth_0.55", _lib.GROWTH_GAMMA)):
        pp = params_g if phys & _lib.GROWTH_GAMMA else params
        tv, _ = timed(lambda pp=pp, phys=phys: angular_cl_device(pp, ell_np, probes, "fp32c", 512, out=cl,
                                                                 physics=phys), args.steps, args.warmup)
        angular_cl_device(pp, ell_np, probes, "fp64", 512, out=c64v, physics=phys)
        angular_cl_device(pp, ell_np, probes, "fp32c", 512, out=cl, physics=phys)
        res["operator_points"][name] = {
            "ms_per_step": tv / args.steps, "cl_per_s": ncl_step / (tv / args.steps * 1e-3),
            "fp32c_max_rel_err_vs_fp64": float(((cl - c64v).abs() / c64v.abs()).max()),
        }
    return res


def accuracy_arm(device):
    """Stated errors of the single-cosmology configurations against the float64
    oracle's stored outputs (tests/golden/c2_oracle.npz, c4_oracle.npz, written
    by tests/golden/make_oracle_fixtures.py; the tests check the same files and
    the live oracle):

    * 10 tracers (5 WL + 5 NC, bias 1.2) x 200 ell in [10, 5000], N = 512: the
      per-spectrum maximum relative error of the FP64 and fp32c C_ell;
    * 5 WL x 50 ell in [10, 3000], fiducial, stored noisy data: the
      log-likelihood (mean and covariance at the cosmology) and its gradient
      over the 8 Cosmology leaves in FP64 and fp32c against the oracle's
      autograd, and against central differences of the FP64 log-likelihood
      (step 1e-5 relative, 1e-5 absolute for zero-valued leaves).
    """
    import torch

    import jax_cosmo_gb300 as jc

    gold = os.path.join(ROOT, "tests", "golden")
    out = {}
    d2 = np.load(os.path.join(gold, "c2_oracle.npz"))
    fid = [float(v) for v in d2["fid"]]
    nz = [jc.redshift.smail_nz(1.0, 2.0, float(z0), gals_per_arcmin2=10.0) for z0 in Z0]
    p2 = [jc.probes.WeakLensing(nz, sigma_e=0.26), jc.probes.NumberCounts(nz, jc.bias.constant_linear_bias(1.2))]
    ref2 = torch.as_tensor(d2["cl"])
    c2 = {"workload": "10 tracers (5 WL + 5 NC, bias 1.2), 55 spectra x 200 ell in [10, 5000], N = 512, fiducial"}
    for prec in ("fp64", "fp32c"):
        cl = jc.cl.angular_cl(jc.Cosmology(*fid), d2["ell"], p2, precision=prec).cpu()
        per = ((cl - ref2) / ref2).abs().amax(dim=1)
        c2[prec] = {"max_rel_err": float(per.max()), "median_rel_err": float(per.median()),
                    "per_spectrum_max_rel_err": [float("%.3g" % v) for v in per.tolist()]}
    out["config_10_tracers"] = c2
    d4 = np.load(os.path.join(gold, "c4_oracle.npz"))
    ell4 = d4["ell"]
    p4 = [jc.probes.WeakLensing(nz, sigma_e=0.26)]
    data = torch.as_tensor(d4["data"], device=device)
    g_o = d4["grad"]
    names = ["Omega_c", "Omega_b", "h", "n_s", "sigma8", "Omega_k", "w0", "wa"]

    def loglike(row, prec="fp64", grad=False):
        ps = {n: torch.tensor(float(v), dtype=torch.float64, requires_grad=grad) for n, v in zip(names, row)}
        c = jc.Cosmology(**ps)
        mu, cov = jc.cl.gaussian_cl_covariance_and_mean(c, ell4, p4, sparse=True, precision=prec)
        ll = jc.likelihood.gaussian_log_likelihood(data, mu, cov)
        if grad:
            ll.backward()
            return float(ll.detach()), np.array([float(ps[n].grad) for n in names])
        return float(ll)

    c4 = {"workload": "5 WL x 50 ell in [10, 3000], N = 512, fiducial; data = mean + seeded noise from its "
                      "covariance; loglike of gaussian_cl_covariance_and_mean + gaussian_log_likelihood",
          "oracle_loglike": float(d4["loglike"])}
    fd = np.zeros(8)
    for i in range(8):
        h = 1e-5 * abs(fid[i]) if fid[i] != 0 else 1e-5
        up, dn = list(fid), list(fid)
        up[i] += h
        dn[i] -= h
        fd[i] = (loglike(up) - loglike(dn)) / (2 * h)
    for prec in ("fp64", "fp32c"):
        ll, g = loglike(fid, prec, True)
        c4[prec] = {"loglike_rel_err": abs(ll - float(d4["loglike"])) / abs(float(d4["loglike"])),
                    "grad_max_err_vs_oracle_autograd": float(np.max(np.abs(g - g_o)) / np.max(np.abs(g_o))),
                    "grad_max_err_vs_fd_fp64": float(np.max(np.abs(g - fd)) / np.max(np.abs(fd))),
                    "grad": [float(v) for v in g]}
    c4["oracle_grad"] = [float(v) for v in g_o]
    c4["err_note"] = ("max |g - g_ref| / max |g_ref| over the 8 leaves; FD: central differences of the FP64 GPU "
                      "log-likelihood, step 1e-5 relative (1e-5 absolute at zero-valued leaves)")
    out["config_gradient"] = c4
    return out


def serving_arm(device, duration_s=10.0, warm_s=3.0, n_chains=64, think_ms=2.0, seed=SEED, n_check=256,
                sweep=((0.0, 5.0), (0.5, 5.0))):
    """64 synthetic HMC chains against the continuous-batching server.

    Each chain (seeded): 1-10 tracers (WeakLensing / NumberCounts mix, smail_nz
    a=1, b=2, z0 in U[0.3, 1.5]), 20-500 log-spaced ell in [10, 5000], data =
    C_ell at its start point (box of the batched workload) with 1% noise,
    covariance fixed at the start point.  A chain submits its next request an
    exponential think time (mean think_ms) after its previous result, its
    parameters jittered by 1% of the box width (Poisson arrivals per chain).
    """
    import heapq
    import queue

    import torch

    import jax_cosmo_gb300 as jc
    from jax_cosmo_gb300 import serving

    lo = np.array([BOX.get(n, (0.0, 0.0))[0] for n in ORDER])
    hi = np.array([BOX.get(n, (0.0, 0.0))[1] for n in ORDER])
    width = hi - lo
    models, pos, rngs = [], [], []
    for c in range(n_chains):
        rng = np.random.default_rng(seed + 1000 + c)
        n_tr = int(rng.integers(1, 11))
        n_wl = int(rng.integers(0, n_tr + 1))
        z0 = rng.uniform(0.3, 1.5, n_tr)
        n_ell = int(rng.integers(20, 501))
        ell = np.logspace(1, np.log10(5000.0), n_ell)
        probes = []
        if n_wl:
            probes.append(jc.probes.WeakLensing([jc.redshift.smail_nz(1.0, 2.0, float(z), gals_per_arcmin2=10.0)
                                                 for z in z0[:n_wl]], sigma_e=0.26))
        if n_tr > n_wl:
            probes.append(jc.probes.NumberCounts([jc.redshift.smail_nz(1.0, 2.0, float(z), gals_per_arcmin2=10.0)
                                                  for z in z0[n_wl:]], jc.bias.constant_linear_bias(1.2)))
        p0 = lo + width * rng.uniform(size=8)
        start = jc.Cosmology(*[float(v) for v in p0])
        mu = jc.cl.angular_cl(start, ell, probes).flatten()
        data = mu * (1.0 + 0.01 * torch.as_tensor(rng.standard_normal(mu.numel()), device=mu.device))
        models.append(serving.ChainModel(probes, ell, data, fiducial=start))
        pos.append(p0)
        rngs.append(rng)
    pos0 = [p.copy() for p in pos]
    st = run_load(device, models, pos, rngs, lo, hi, width, think_ms, duration_s, warm_s, n_check)
    st["load_sweep"] = []
    for tm, dur in sweep:
        pos = [p.copy() for p in pos0]
        s2 = run_load(device, models, pos, rngs, lo, hi, width, tm, dur, 2.0, 0)
        st["load_sweep"].append({"think_ms_mean": tm, "duration_s": dur, "requests_per_s": s2["requests_per_s"],
                                 "p50_ms": s2["p50_ms"], "p99_ms": s2["p99_ms"], "mean_batch": s2["mean_batch"],
                                 "max_batch": s2["max_batch"], "completed": s2["completed"]})
    st.update({"chains": n_chains, "think_ms_mean": think_ms, "duration_s": duration_s,
               "tracers_per_chain": [int(m.g.n_tracers) for m in models],
               "n_ell_per_chain": [int(m.n_ell) for m in models], "precision": "fp32c", "dtype": "f32c+f64"})
    return st


def run_load(device, models, pos, rngs, lo, hi, width, think_ms, duration_s, warm_s, n_check):
    """One load point: each chain submits its next request an exponential
    think time (mean think_ms; 0 = at once) after its previous result."""
    import heapq
    import queue

    import torch

    import jax_cosmo_gb300 as jc
    from jax_cosmo_gb300 import serving

    n_chains = len(models)
    done_q = queue.Queue()
    srv = serving.Server(device=device, hbm_budget=8 << 30, max_batch=256, n_streams=2).start()

    def think(c):
        return rngs[c].exponential(think_ms * 1e-3) if think_ms > 0 else 0.0

    def submit(c):
        step = rngs[c].normal(0.0, 0.01, 8) * width
        pos[c] = np.clip(pos[c] + step, lo, hi)
        f = srv.submit(models[c], pos[c])
        f.add_done_callback(lambda _f, c=c: done_q.put(c))
        return f

    heap = [(time.perf_counter() + think(c), c) for c in range(n_chains)]
    heapq.heapify(heap)
    t_start = time.perf_counter()
    t_measure = t_start + warm_s
    t_end = t_measure + duration_s
    reset = False
    sample = []
    while True:
        now = time.perf_counter()
        if not reset and now >= t_measure:
            srv.reset_stats()
            reset = True
        if now >= t_end:
            break
        while heap and heap[0][0] <= now:
            _, c = heapq.heappop(heap)
            f = submit(c)
            if reset and len(sample) < n_check:
                sample.append((c, pos[c].copy(), f))
        timeout = max(0.0, heap[0][0] - now) if heap else 0.01
        try:
            c = done_q.get(timeout=min(timeout, 0.01))
            heapq.heappush(heap, (time.perf_counter() + think(c), c))
            while True:
                c = done_q.get_nowait()
                heapq.heappush(heap, (time.perf_counter() + think(c), c))
        except queue.Empty:
            pass
    st = srv.stats()
    srv.stop()
    if not sample:
        return st
    # served log-likelihoods and gradients against the plain float64 method
    # (public API: angular_cl_jacobian in FP64, then -J^T P r), every sampled request
    err_ll, err_g, err_gs = [], [], []
    for c, p, f in sample:
        r = f.result()
        m = models[c]
        cl, jac = jc.autodiff.angular_cl_jacobian(jc.Cosmology(*[float(v) for v in p]), m.ell, m.probes)
        res = (cl.flatten() - m.data).reshape(m.n_cls, m.n_ell)
        pr = torch.einsum("lpq,ql->pl", m.prec, res)
        ll = -0.5 * float((res * pr).sum())
        g = -torch.einsum("pld,pl->d", jac, pr).cpu().numpy()
        err_ll.append(abs(r.loglike - ll) / abs(ll))
        err_g.append(float(np.max(np.abs(np.asarray(r.grad) - g)) / np.max(np.abs(g))))
        gs = torch.einsum("pld,pl->d", jac.abs(), pr.abs()).cpu().numpy()
        err_gs.append(float(np.max(np.abs(np.asarray(r.grad) - g) / gs)))
    st["accuracy_vs_fp64"] = {
        "checked_requests": len(sample),
        "loglike_max_rel_err": float(max(err_ll)), "loglike_median_rel_err": float(np.median(err_ll)),
        "grad_max_err": float(max(err_g)), "grad_median_err": float(np.median(err_g)),
        "grad_scaled_max_err": float(max(err_gs)), "grad_scaled_median_err": float(np.median(err_gs)),
        "grad_err_note": "grad_max_err: max |g - g64| / max |g64| over the 8 Cosmology leaves, per request "
                         "(large where the gradient cancels near a chain's maximum); grad_scaled: "
                         "max_d |g_d - g64_d| / sum_{p,l} |J64_pld| |(P r)_pl|, the error against the size of "
                         "the summed terms",
        "reference": "public API in float64: angular_cl_jacobian, then logL = -r^T P r / 2, grad = -J^T P r"}
    return st


def measure_peaks(device):
    """FP64 FMA and MUFU ex2 issue peaks of this GPU (calibration kernels of libjcg)."""
    import ctypes

    import torch

    from jax_cosmo_gb300 import _lib

    sms = torch.cuda.get_device_properties(device).multi_processor_count
    blocks = sms * 8
    st = _lib.stream_of(device)
    out64 = torch.empty(blocks * 256, dtype=torch.float64, device=device)
    out32 = torch.empty(blocks * 256, dtype=torch.float32, device=device)
    res = {}
    for name, fn, buf, iters in (("fp64", "jcg_calib_peak_fp64", out64, 200), ("mufu", "jcg_calib_peak_mufu", out32, 4000)):
        for _ in range(2):
            _lib.call(fn, _lib.ptr(buf), blocks, iters, st)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _lib.call(fn, _lib.ptr(buf), blocks, iters, st)
        e1.record()
        e1.synchronize()
        ops = blocks * 256 * iters * 128
        res[name] = ops / (e0.elapsed_time(e1) * 1e-3)
    return {"fp64_tflops": 2.0 * res["fp64"] / 1e12, "dfma_per_s": res["fp64"], "mufu_per_s": res["mufu"],
            "sm_count": sms, "how": "libjcg calibration kernels: 8 chains x 16 unrolled DFMA / ex2.approx per "
                                   "iteration, SMs x 8 blocks x 256 threads, CUDA events"}


def _issue_peak(res):
    mhz = (res.get("clocks") or {}).get("sm_mhz") or 2070.0
    return 4 * res.get("sm_count", 152) * mhz * 1e6


def rooflines(res, B, live):
    """Per-kernel rooflines of the fp32c step; the dominant kernel first."""
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    stages = res["stages_ms"]
    peak_issue = _issue_peak(res)
    out = {}
    for k, ms in stages.items():
        t = ms * 1e-3
        e = {"kernel": KERNEL_NAMES.get(k, k), "ms": ms}
        if k in ALG_BYTES:
            e["algorithmic_bytes_per_launch"] = ALG_BYTES[k] * B
            e["hbm_frac"] = ALG_BYTES[k] * B / t / 1e9 / hbm
        if k in TRAFFIC_PER_COSMO:
            e["traffic"] = TRAFFIC_PER_COSMO[k] * B
            if k in TRAFFIC_NOTE:
                e["traffic_note"] = TRAFFIC_NOTE[k]
        if k in FP64_OPS:
            ach = FP64_OPS[k] * B / t / 1e12
            e["fp64"] = {"achieved": ach, "peak": live["fp64_tflops"], "unit": "TFLOP/s",
                         "frac": ach / live["fp64_tflops"], "peak_source": "measured live (calibration kernel)"}
        if k == "limber":
            # issue-bound: every pipe below half busy
            nodes = B * N_ELL * 513
            ach = nodes * WARP_INSTR_PER_NODE / t
            mufu = nodes * MUFU_PER_NODE / t
            e.update({"bound": "issue", "achieved": ach / 1e9, "peak": peak_issue / 1e9, "unit": "Gwarp-instr/s",
                      "frac": ach / peak_issue, "warp_instr_per_node": WARP_INSTR_PER_NODE,
                      "peak_source": "4 warp instructions per SM per clock x SMs x sampled SM clock",
                      "sfu": {"achieved_gmufu_s": mufu / 1e9, "peak_gmufu_s": live["mufu_per_s"] / 1e9,
                              "frac": mufu / live["mufu_per_s"], "mufu_per_node": MUFU_PER_NODE,
                              "peak_source": "measured live (calibration kernel)"}})
        elif k in WARP_INSTR_PER_COSMO:
            ach = WARP_INSTR_PER_COSMO[k] * B / t
            e.update({"bound": "issue", "achieved": ach / 1e9, "peak": peak_issue / 1e9, "unit": "Gwarp-instr/s",
                      "frac": ach / peak_issue, "warp_instr_per_cosmology": WARP_INSTR_PER_COSMO[k],
                      "peak_source": "4 warp instructions per SM per clock x SMs x sampled SM clock"})
        out[k] = e
    dom = max(stages, key=lambda k: stages[k])
    return dom, out


def vjp_rooflines(stages_ms, B, res):
    """Per-stage rooflines of the fp32c vector-Jacobian product (all bound by
    instruction issue and latency; HBM fractions beside)."""
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    peak_issue = _issue_peak(res)
    out = {}
    for k, ms in stages_ms.items():
        t = ms * 1e-3
        ach = VJP_WARP_INSTR_PER_COSMO[k] * B / t
        e = {"ms": ms, "bound": "issue", "achieved": ach / 1e9, "peak": peak_issue / 1e9, "unit": "Gwarp-instr/s",
             "frac": ach / peak_issue, "warp_instr_per_cosmology": VJP_WARP_INSTR_PER_COSMO[k],
             "algorithmic_bytes_per_launch": VJP_ALG_BYTES[k] * B,
             "hbm_frac": VJP_ALG_BYTES[k] * B / t / 1e9 / hbm, "traffic": VJP_TRAFFIC_PER_COSMO[k] * B}
        if k == "product":
            nodes = B * N_ELL * 513
            e["warp_instr_per_node"] = VJP_PRODUCT_WARP_INSTR_PER_NODE
            e["mufu_per_node"] = VJP_PRODUCT_MUFU_PER_NODE
            e["kernel"] = "grad_vjp32_kernel<0, 0>"
            e["gnodes_per_s"] = nodes / t / 1e9
        out[k] = e
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=B_DEFAULT)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=10.0)
    ap.add_argument("--jacobian-only", action="store_true",
                    help="time only the fp32c C_ell + Jacobian of the batch (profiling)")
    ap.add_argument("--fwd-only", action="store_true",
                    help="time only the fp32c C_ell step of the batch (profiling)")
    ap.add_argument("--vjp-only", action="store_true",
                    help="time only the fp32c C_ell + vector-Jacobian product of the batch (profiling)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    config = {"workload": "batched angular_cl: 4096 cosmologies x 5 WL bins x 100 ell (15 spectra), N=512",
              "n_cosmo_per_gpu": args.batch, "n_tracers": 5, "n_cls": 15, "n_ell": N_ELL,
              "n_limber": 512, "ell_range": [20, 3000], "seed": SEED,
              "l2": "flushed (256 MB write) between timed steps", "parallelism": f"replicas x{args.gpus}"}

    if args.impl == "reference":
        if rank != 0:
            return
        P = draw_params(args.batch)
        vals = []
        for _ in range(args.warmup):
            cpu_baseline(P, budget_s=2.0)
        cb = None
        for _ in range(args.steps):
            cb = cpu_baseline(P, budget_s=max(3.0, 30.0 / max(args.steps, 1)))
            vals.append(cb["value"])
        v = float(np.median(vals))
        print(json.dumps({
            "impl": "reference",
            "metric": "C_ell evals/s batched vs plain at \u22641e-4 rel err; p50/p99 loglike+grad latency",
            "value": v,
            "unit": "C_ell/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config,
            "cpu_baseline": {**cb, "value": v},
            "e2e": {"value": v, "unit": "C_ell/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference JAX CPU path unavailable on this host (no jax); the float64 oracle "
                    "port of the path is timed with one process per core",
        }))
        return

    cb = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # spawn pool before the first CUDA call
        cb = cpu_baseline(draw_params(args.batch), budget_s=12.0)

    import torch

    if world > 1:
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    res = gpu_arm(args, rank, world, device)
    if "jacobian_only" in res:
        if rank == 0:
            print(json.dumps(res["jacobian_only"]))
        return
    acc = accuracy_arm(device) if rank == 0 else None
    serve = None
    if rank == 0 and not args.no_serving:
        serve = serving_arm(device, duration_s=args.serve_seconds)
    if rank != 0:
        return
    K = res["K"]
    ms = res["t_fast"] / K
    value = res["ncl_step"] * world / (ms * 1e-3)
    fp64_value = res["ncl_step"] * world / (res["t64"] / res["n64"] * 1e-3)
    e2e = res["ncl_step"] * world / (res["t_e2e"] / K * 1e-3)
    live = measure_peaks(device)
    dom, rls = rooflines(res, args.batch, live)
    rl = dict(rls[dom])
    plain = res["plain_fp64_single"]["cl_per_s"]
    jac = res["jacobian"]
    for prec in jac:
        jac[prec]["over_plain_fp64_single"] = jac[prec]["cl_grad_per_s"] / plain
    out = {
        "metric": "C_ell evals/s batched vs plain at \u22641e-4 rel err; p50/p99 loglike+grad latency",
        "value": value, "unit": "C_ell/s", "n_gpus": world, "steps": K, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32c+f64", "data": "synthetic", "config": config,
        "fp64_value": fp64_value, "fp32c_over_fp64": value / fp64_value,
        "plain_fp64_single": res["plain_fp64_single"],
        "batched_over_plain_fp64_single": value / plain,
        "cl_grad": jac,
        "operator_points": res["operator_points"],
        "loglike_grad_latency_ms": ({"p50": serve["p50_ms"], "p99": serve["p99_ms"]} if serve else None),
        "serving": serve,
        "fp32c_max_rel_err_vs_fp64": res["fp32c_max_rel_err_vs_fp64"],
        "accuracy": acc,
        "cosmologies_per_s": value / 1500.0,
        "e2e": {"value": e2e, "unit": "C_ell/s", "h2d_bytes_per_step": res["h2d"],
                "d2h_bytes_per_step": res["d2h"]},
        "gpu_launches": 5 * K,
        "stage_ms": res["stages_ms"],
        "roofline": rl, "rooflines": rls, "peaks_live": live,
        "clocks": res["clocks"],
        "cpu_baseline": cb,
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
