"""Serving loop: continuous batching of log-likelihood + gradient requests.

Sampler chains (HMC, NUTS) each hold a likelihood of their own: a set of
probes, an ell grid, a data vector and a covariance, i.e. the reference's

    mu = angular_cl(cosmo, ell, probes)                   angular_cl.py:49-98
    logL = gaussian_log_likelihood(data, mu, C)           likelihood.py:9-61
    grad = jax.grad(logL)(cosmo)                          README.md:14-27

with the covariance held fixed (the intro notebook's likelihood).  A chain
registers once as a ``ChainModel``: its geometry (n(z) grids, Limber nodes,
ell), its data vector and its inverse covariance blocks stay resident in HBM.
It then submits ``(model, parameters)`` requests to a ``Server``, which

* admits pending requests in arrival order while their workspace footprint
  fits in the free part of a fixed HBM arena (``hbm_budget`` bytes);
* runs every admitted request, whatever its tracer count and ell grid, in one
  launch sequence (``jcg_requests_run``, mode LOGLIKE_GRAD: tables with
  tangents, halofit rows, radial kernels, the Limber Jacobian, then logL and
  its gradient over the 8 Cosmology leaves; ``precision`` "fp32c" -- float64
  tables, float32 Limber integrand and lensing kernels with compensated sums --
  or "fp64");
* keeps up to ``n_streams`` such batches on the GPU at once, each on its own
  CUDA stream, so that requests arriving while a batch runs are admitted and
  launched as soon as a stream slot and arena space are free (their work
  overlaps on the device);
* returns each result through a ``concurrent.futures.Future`` and records its
  latency (submit -> result) for p50 / p99.

Each request's result depends only on its own inputs (per-request CTAs and
fixed-order sums), so it is the same alone and in any mix.

Failure handling is on the host: a request whose footprint exceeds the arena
is refused at submit (``MemoryError``), non-finite parameters are refused
(``ValueError``), a cancelled future is skipped at admission, a library error
fails the futures of its batch, and a batch not done within ``timeout_s`` fails
with ``TimeoutError`` (its stream slot and arena space are then retired, since
the device may still write to them).
"""
from __future__ import annotations

import collections
import ctypes
import threading
import time
from concurrent.futures import Future

import numpy as np
import torch

from jax_cosmo_gb300 import _geometry, _lib
from jax_cosmo_gb300 import sparse as sparse_mod

__all__ = ["ChainModel", "Server", "ServeResult"]

ServeResult = collections.namedtuple("ServeResult", ["loglike", "grad"])

_ALIGN = 256


def _round(n):
    return (int(n) + _ALIGN - 1) // _ALIGN * _ALIGN


class ChainModel:
    """Device-resident likelihood of one chain.

    ``cov`` is the sparse covariance [n_cls, n_cls, n_ell] (block diagonal in
    ell, angular_cl.py:120-163); if None it is the Gaussian covariance with
    noise at ``fiducial`` (default Planck15), f_sky given.  ``data`` has length
    n_cls * n_ell in (cls, ell) order, like the reference's flattened mean.
    """

    def __init__(self, probes, ell, data, cov=None, *, fiducial=None, f_sky=0.25, n_limber=512,
                 device=None, transfer_fn=None, nonlinear_fn=None):
        from jax_cosmo_gb300 import angular_cl as cl_mod
        from jax_cosmo_gb300 import power, transfer
        from jax_cosmo_gb300.parameters import Planck15

        tf = transfer_fn or transfer.Eisenstein_Hu
        nl = nonlinear_fn or power.halofit
        physics = cl_mod.physics_code(tf, nl)
        self.device = _lib.require_cuda(device)
        self.probes = probes
        self.ell = _geometry.ell_host(ell)
        self.g, self.geo, _ = _geometry.get_geometry(probes, self.ell, n_limber, self.device, physics)
        self.n_cls = _geometry.n_cls_of(self.g)
        self.n_ell = int(self.g.n_ell)
        N = self.n_cls * self.n_ell
        self.data = torch.as_tensor(np.asarray(data, dtype=np.float64) if not isinstance(data, torch.Tensor)
                                    else data.detach(), dtype=torch.float64).to(self.device).reshape(-1)
        if self.data.numel() != N:
            raise ValueError(f"data has {self.data.numel()} entries, expected n_cls * n_ell = {N}")
        if cov is None:
            cosmo = fiducial if fiducial is not None else Planck15()
            _, cov = cl_mod.gaussian_cl_covariance_and_mean(cosmo, self.ell, probes, tf, nl, f_sky=f_sky,
                                                            sparse=True, n_limber=n_limber)
        cov = torch.as_tensor(cov, dtype=torch.float64).to(self.device)
        if cov.shape != (self.n_cls, self.n_cls, self.n_ell):
            raise ValueError(f"covariance {tuple(cov.shape)}: expected sparse {(self.n_cls, self.n_cls, self.n_ell)}")
        # per-ell inverse blocks as [n_ell, n_cls, n_cls] (libjcg's sparse.inv;
        # its block limit, 160, is above the 136 spectra of 16 tracers)
        self.prec = sparse_mod.inv(cov).permute(2, 0, 1).contiguous()
        self.resident_bytes = (self.geo.numel() * self.geo.element_size() + self.data.numel() * 8
                               + self.prec.numel() * 8)
        self._addr = (ctypes.addressof(self.g), self.geo.data_ptr(), self.data.data_ptr(),
                      self.prec.data_ptr())
        table = np.zeros(1, _lib.REQUEST_DTYPE)
        self._fill(table, 0, self.geo.data_ptr(), self.data.data_ptr())
        # workspace share of one request (no a-splits), additive over a batch;
        # the larger of the two precisions
        self.footprint = 0
        for prec in (_lib.FP64, _lib.FP32C):
            lo, hi = ctypes.c_size_t(), ctypes.c_size_t()
            _lib.call("jcg_requests_workspace_size", ctypes.c_void_p(table.ctypes.data), 1,
                      _lib.REQ_LOGLIKE_GRAD, prec, ctypes.byref(lo), ctypes.byref(hi))
            self.footprint = max(self.footprint, _round(lo.value))

    def _fill(self, table, i, params_ptr, out_ptr):
        g, geo, data, prec = self._addr
        table[i] = (g, geo, params_ptr, 0, 0, data, prec, out_ptr)


class _Arena:
    """First-fit byte ranges of one fixed HBM buffer (offsets 256-byte aligned)."""

    def __init__(self, size):
        self.size = int(size) // _ALIGN * _ALIGN
        self.free = [(0, self.size)]
        self.used = 0
        self.peak = 0

    def largest(self):
        return max((n for _, n in self.free), default=0)

    def alloc(self, n):
        n = _round(n)
        for k, (off, length) in enumerate(self.free):
            if length >= n:
                if length == n:
                    self.free.pop(k)
                else:
                    self.free[k] = (off + n, length - n)
                self.used += n
                self.peak = max(self.peak, self.used)
                return off
        return None

    def release(self, off, n):
        n = _round(n)
        self.used -= n
        self.free.append((off, n))
        self.free.sort()
        merged = []
        for o, length in self.free:
            if merged and merged[-1][0] + merged[-1][1] == o:
                merged[-1] = (merged[-1][0], merged[-1][1] + length)
            else:
                merged.append((o, length))
        self.free = merged


class _CudaBackend:
    """One CUDA stream, pinned staging and device slots per batch slot."""

    def __init__(self, device, arena_bytes, n_streams, max_batch, precision, trace=False):
        self.device = _lib.require_cuda(device)
        self.trace = trace
        self.trace_log = []  # (slot, start event, end event) of every launch when tracing
        self.precision = precision
        self.arena = torch.empty(max(int(arena_bytes), _ALIGN), dtype=torch.uint8, device=self.device)
        self.streams = [torch.cuda.Stream(self.device) for _ in range(n_streams)]
        self.events = [None] * n_streams
        self.params_host = [torch.empty(max_batch, 8, dtype=torch.float64).pin_memory() for _ in range(n_streams)]
        self.out_host = [torch.empty(max_batch, 9, dtype=torch.float64).pin_memory() for _ in range(n_streams)]
        self.params_dev = [torch.empty(max_batch, 8, dtype=torch.float64, device=self.device)
                           for _ in range(n_streams)]
        self.out_dev = [torch.empty(max_batch, 9, dtype=torch.float64, device=self.device)
                        for _ in range(n_streams)]
        self.tables = [np.zeros(max_batch, _lib.REQUEST_DTYPE) for _ in range(n_streams)]
        self.launches = 0

    def plan(self, models):
        """(bytes without a-splits, bytes with the splits that fill the GPU)."""
        table = np.zeros(len(models), _lib.REQUEST_DTYPE)
        for i, m in enumerate(models):
            m._fill(table, i, m.geo.data_ptr(), m.data.data_ptr())
        lo, hi = ctypes.c_size_t(), ctypes.c_size_t()
        _lib.call("jcg_requests_workspace_size", ctypes.c_void_p(table.ctypes.data), len(models),
                  _lib.REQ_LOGLIKE_GRAD, self.precision, ctypes.byref(lo), ctypes.byref(hi))
        return lo.value, hi.value

    def launch(self, slot, reqs, off, nbytes):
        n = len(reqs)
        s = self.streams[slot]
        ph, pd = self.params_host[slot], self.params_dev[slot]
        ph.numpy()[:n] = np.stack([r.params for r in reqs])
        table = self.tables[slot]
        p0, o0 = pd.data_ptr(), self.out_dev[slot].data_ptr()
        for i, r in enumerate(reqs):
            r.model._fill(table, i, p0 + 64 * i, o0 + 72 * i)
        with torch.cuda.stream(s):
            if self.trace:
                e0 = torch.cuda.Event(enable_timing=True)
                e0.record(s)
            pd[:n].copy_(ph[:n], non_blocking=True)
            _lib.call("jcg_requests_run", ctypes.c_void_p(table.ctypes.data), n, _lib.REQ_LOGLIKE_GRAD,
                      self.precision, ctypes.c_void_p(self.arena.data_ptr() + off), ctypes.c_size_t(nbytes),
                      ctypes.c_void_p(s.cuda_stream))
            self.out_host[slot][:n].copy_(self.out_dev[slot][:n], non_blocking=True)
            ev = torch.cuda.Event(enable_timing=self.trace)
            ev.record(s)
            if self.trace:
                self.trace_log.append((slot, e0, ev))
        self.events[slot] = ev
        self.launches += 1

    def ready(self, slot):
        return self.events[slot].query()

    def fetch(self, slot, n):
        return self.out_host[slot][:n].numpy().copy()


class _Req:
    __slots__ = ("model", "params", "future", "t_submit")

    def __init__(self, model, params, future, t_submit):
        self.model = model
        self.params = params
        self.future = future
        self.t_submit = t_submit


class _Flight:
    __slots__ = ("reqs", "off", "nbytes", "t_launch")

    def __init__(self, reqs, off, nbytes, t_launch):
        self.reqs = reqs
        self.off = off
        self.nbytes = nbytes
        self.t_launch = t_launch


class Server:
    """Continuous-batching server for ``ChainModel`` likelihood + gradient requests.

    ``submit(model, params)`` returns a Future resolving to
    ``ServeResult(loglike, grad[8])`` (gradient over Omega_c, Omega_b, h, n_s,
    sigma8, Omega_k, w0, wa).  Use as a context manager or call ``start`` /
    ``stop``.
    """

    def __init__(self, device=None, hbm_budget=1 << 30, max_batch=512, n_streams=2, timeout_s=60.0,
                 poll_s=50e-6, precision="fp32c", backend=None, trace=False):
        from jax_cosmo_gb300.angular_cl import _precision_code

        if n_streams < 1 or max_batch < 1:
            raise ValueError("n_streams and max_batch must be >= 1")
        self.precision = precision
        prec = _precision_code(precision)
        self.max_batch = int(max_batch)
        self.timeout_s = float(timeout_s)
        self.poll_s = float(poll_s)
        self._arena = _Arena(hbm_budget)
        self._backend = backend if backend is not None else _CudaBackend(device, self._arena.size, n_streams,
                                                                          self.max_batch, prec, trace)
        self._slots = [None] * n_streams
        self._dead = [False] * n_streams
        self._pending = collections.deque()
        self._cv = threading.Condition()
        self._stop = False
        self._thread = None
        self._lat = []
        self._batch_sizes = []
        self._completed = 0
        self._failed = 0
        self._t_first = None
        self._t_last = None

    # ------------------------------------------------------------ client ----
    def submit(self, model, params):
        p = np.asarray(params, dtype=np.float64).reshape(-1)
        if p.size != 8:
            raise ValueError("params: the 8 Cosmology leaves (Omega_c, Omega_b, h, n_s, sigma8, Omega_k, w0, wa)")
        if not np.all(np.isfinite(p)):
            raise ValueError("Cosmology parameters must be finite")
        if model.footprint > self._arena.size:
            raise MemoryError(f"request needs {model.footprint} bytes of workspace, the arena has {self._arena.size}")
        fut = Future()
        req = _Req(model, p.copy(), fut, time.perf_counter())
        with self._cv:
            if self._stop:
                raise RuntimeError("server is stopped")
            self._pending.append(req)
            self._cv.notify()
        return fut

    def start(self):
        if self._thread is None:
            self._thread = threading.Thread(target=self._loop, name="jcg-serve", daemon=True)
            self._thread.start()
        return self

    def stop(self, wait=True):
        with self._cv:
            self._stop = True
            self._cv.notify()
        if wait and self._thread is not None:
            self._thread.join()

    def __enter__(self):
        return self.start()

    def __exit__(self, *exc):
        self.stop()

    def device_intervals(self):
        """With ``trace=True``: (stream slot, start ms, end ms) of every launched
        batch on the GPU's clock (CUDA events around the batch's copies and
        kernels on its stream), relative to the first batch's start.  Call
        after ``stop``."""
        log = getattr(self._backend, "trace_log", [])
        if not log:
            return []
        for _, _, e1 in log:
            e1.synchronize()
        ref = log[0][1]
        return [(slot, ref.elapsed_time(e0), ref.elapsed_time(e1)) for slot, e0, e1 in log]

    def reset_stats(self):
        """Forget latencies and counts so far (e.g. after a warm-up period)."""
        self._lat = []
        self._batch_sizes = []
        self._completed = 0
        self._failed = 0
        self._t_first = time.perf_counter()
        self._t_last = None

    def stats(self):
        lat = np.asarray(self._lat)
        span = (self._t_last - self._t_first) if self._completed and self._t_last and self._t_last > self._t_first else 0.0
        return {
            "completed": self._completed,
            "failed": self._failed,
            "batches": len(self._batch_sizes),
            "mean_batch": float(np.mean(self._batch_sizes)) if self._batch_sizes else 0.0,
            "max_batch": int(max(self._batch_sizes)) if self._batch_sizes else 0,
            "p50_ms": float(np.percentile(lat, 50) * 1e3) if lat.size else None,
            "p99_ms": float(np.percentile(lat, 99) * 1e3) if lat.size else None,
            "mean_ms": float(lat.mean() * 1e3) if lat.size else None,
            "requests_per_s": self._completed / span if span > 0 else None,
            "arena_bytes": self._arena.size,
            "arena_peak_bytes": self._arena.peak,
        }

    # ------------------------------------------------------------ server ----
    def _loop(self):
        while True:
            reaped = self._reap()
            launched = self._admit()
            with self._cv:
                busy = any(s is not None for s in self._slots)
                if self._stop and not self._pending and not busy:
                    return
                if not reaped and not launched:
                    self._cv.wait(self.poll_s if busy else 0.05)

    def _take(self):
        """Pending requests (arrival order) that fit in the largest free arena range."""
        batch, total = [], 0
        room = self._arena.largest()
        with self._cv:
            while self._pending and len(batch) < self.max_batch:
                req = self._pending[0]
                if req.future.cancelled():
                    self._pending.popleft()
                    continue
                fp = req.model.footprint
                if total + fp > room:
                    break
                self._pending.popleft()
                if not req.future.set_running_or_notify_cancel():
                    continue
                batch.append(req)
                total += fp
        return batch, total

    def _admit(self):
        launched = False
        for slot in range(len(self._slots)):
            if self._slots[slot] is not None or self._dead[slot]:
                continue
            batch, total = self._take()
            if not batch:
                break
            try:
                lo, hi = self._backend.plan([r.model for r in batch])
            except Exception as e:  # noqa: BLE001 - delivered to the callers
                self._fail(batch, e)
                continue
            need = hi if self._arena.largest() >= hi else max(lo, total)
            off = self._arena.alloc(need)
            if off is None:
                need = lo
                off = self._arena.alloc(need)
            if off is None:  # cannot happen: total >= lo fits the largest free range
                self._fail(batch, MemoryError("arena fragmentation"))
                continue
            try:
                self._backend.launch(slot, batch, off, need)
            except Exception as e:  # noqa: BLE001 - delivered to the callers
                self._arena.release(off, need)
                self._fail(batch, e)
                continue
            now = time.perf_counter()
            if self._t_first is None:
                self._t_first = min(r.t_submit for r in batch)
            self._slots[slot] = _Flight(batch, off, need, now)
            self._batch_sizes.append(len(batch))
            launched = True
        return launched

    def _reap(self):
        reaped = False
        for slot, fl in enumerate(self._slots):
            if fl is None:
                continue
            if self._backend.ready(slot):
                out = self._backend.fetch(slot, len(fl.reqs))
                self._arena.release(fl.off, fl.nbytes)
                self._slots[slot] = None
                now = time.perf_counter()
                for i, r in enumerate(fl.reqs):
                    self._lat.append(now - r.t_submit)
                    r.future.set_result(ServeResult(float(out[i, 0]), out[i, 1:9].copy()))
                self._completed += len(fl.reqs)
                self._t_last = now
                reaped = True
            elif time.perf_counter() - fl.t_launch > self.timeout_s:
                # the device may still write this slot's buffers: retire both
                self._slots[slot] = None
                self._dead[slot] = True
                self._fail(fl.reqs, TimeoutError(f"batch not done after {self.timeout_s} s"))
                reaped = True
        if all(self._dead):
            with self._cv:
                pend = list(self._pending)
                self._pending.clear()
            self._fail([r for r in pend if r.future.set_running_or_notify_cancel()],
                       RuntimeError("no usable stream slot left"))
        return reaped

    def _fail(self, reqs, exc):
        for r in reqs:
            if not r.future.done():
                r.future.set_exception(exc)
        self._failed += len(reqs)


def angular_cl_ragged(items, precision="fp32c", n_limber=512, device=None):
    """C_ell of several (cosmology, ell, probes) triples in one launch sequence.

    Each triple may have its own probes (tracer count, n(z)) and ell grid; the
    result is a list of [n_cls, n_ell] float64 tensors, each the same as
    ``angular_cl(cosmology, ell, probes)`` alone.
    """
    from jax_cosmo_gb300.angular_cl import _precision_code

    prec = _precision_code(precision)
    device = _lib.require_cuda(device)
    items = list(items)
    n = len(items)
    if n == 0:
        return []
    params = torch.empty(n, 8, dtype=torch.float64, device=device)
    table = np.zeros(n, _lib.REQUEST_DTYPE)
    outs, keep = [], []
    for i, (cosmo, ell, probes) in enumerate(items):
        if cosmo.batch_size is not None:
            raise ValueError("angular_cl_ragged takes one cosmology per item")
        if cosmo.physics_bits():
            raise NotImplementedError("angular_cl_ragged takes cosmologies without gamma growth")
        g, geo, _ = _geometry.get_geometry(probes, _geometry.ell_host(ell), n_limber, device)
        params[i] = cosmo.param_tensor(device)[0]
        out = torch.empty(_geometry.n_cls_of(g), g.n_ell, dtype=torch.float64, device=device)
        outs.append(out)
        keep.append((g, geo))
        table[i] = (ctypes.addressof(g), geo.data_ptr(), params.data_ptr() + 64 * i, out.data_ptr(), 0, 0, 0, 0)
    lo, hi = ctypes.c_size_t(), ctypes.c_size_t()
    tp = ctypes.c_void_p(table.ctypes.data)
    _lib.call("jcg_requests_workspace_size", tp, n, _lib.REQ_CL, prec, ctypes.byref(lo), ctypes.byref(hi))
    ws = _lib.workspace(hi.value, device)
    _lib.call("jcg_requests_run", tp, n, _lib.REQ_CL, prec, _lib.ptr(ws), ctypes.c_size_t(ws.numel()),
              _lib.stream_of(device))
    del keep
    return outs
