"""Benchmark of the Krylov hot path on one GB300 (or N replicas).

Workload (default): 3-D variable-coefficient diffusion on a 256^3 grid
(16,777,216 rows, 117,047,296 nonzeros), log-normal cell coefficients
(sigma = 1, seed 2) with harmonic face averaging, RHS U[-1, 1] (seed 3),
Jacobi-preconditioned CG to rtol 1e-8, zero initial guess.  A "step" is one
full solve.  The headline `value` is the time-to-rtol of the mixed-precision
refined PCG: FP64 iterations until the residual is below 3e-3 ||b|| (the
first decades, where the solution's large components form), then FP32
recurrences with FP64 residual replacement, FP64 update and FP64 stopping
test.  That solve ends within 1e-8 of the FP64 PCG's iterate; the same
solver with FP32 recurrences from the first iteration is timed too, with
its distance.  The plain FP64 GPU PCG is timed the same way and their
ratio is reported, with every result's forward error against a tight FP64
solve (rtol 1e-12).

The matrix (1.7 GB FP64) is larger than L2 (129 MB), so no flush is needed
between steps.  Timing: CUDA events on the library's stream around exactly
K steps, after W warm-up steps, with nvidia-smi clock sampling during the
timed region.  `e2e` times the same solve through the public C ABI with the
right-hand side uploaded from pinned host memory and the solution downloaded
every step.

`--impl reference` runs ONE complete solve of the reference's own serial
Jacobi-PCG (its unmodified templates, compiled by `make -C oracle ref` into
oracle/_ref/ref_driver; without that build, the oracle restatement pinned
bit-exact to it) on the host, one core (the reference's serial path), with a
time stamp at every iteration.  Its W + K steps are W + K consecutive chunks
of that solve's iterations (the first chunk includes the set-up); the
`value` is the measured wall time of the whole solve.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "PCG time-to-rtol1e-8 & SpMV HBM GB/s; mixed-prec vs FP64 speedup, 1 GB300"


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(values, ws):
    """The element-wise maximum of `values` over the ranks of the process
    group (every rank gets it); `values` unchanged on one rank.  The replicas'
    per-step times are combined this way: the job takes as long as its
    slowest rank."""
    if ws <= 1:
        return list(values)
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(values), dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t]


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


CODING_NAMES = {0: "colids", 1: "patterns", 2: "symmetric", 3: "grid", 4: "grid_general"}


def spmv_bytes(nrows, nnz, val_bytes, coding=0, nblk=0, nsym=3):
    """Algorithmic bytes of one CSR SpMV: the matrix data of the format, x
    read once, y written once.  Column ids (coding 0): values + int32 column
    per nonzero + int32 row offsets.  Row patterns (1): values + one
    pattern-id byte per row + 16 bytes of warp offsets per 256-row block.
    Symmetric storage (2): the diagonal and `nsym` upper diagonals (3 for a
    7-point operator) + one pattern-id byte per row.  Pattern tables (<= 8 KB)
    are read once per CTA out of L2 and not counted.  Grid stencil (3): the
    diagonal and upper diagonals only (rows addressed by grid coordinates);
    general grid stencil (4): the diagonal, upper and lower diagonals."""
    if coding == 0:
        mat = nnz * val_bytes + 4 * nnz + 4 * (nrows + 1)
    elif coding == 1:
        mat = nnz * val_bytes + nrows + 16 * nblk
    elif coding == 2:
        mat = (nsym + 1) * nrows * val_bytes + nrows
    elif coding == 4:
        mat = (2 * nsym + 1) * nrows * val_bytes
    else:
        mat = (nsym + 1) * nrows * val_bytes
    return mat + 2 * nrows * val_bytes


def gmres_solve_bytes(nrows, nnz, coding, nblk, iters, restarts, m=30, ortho="cgs2",
                      basis_bytes=4):
    """Algorithmic bytes of a right-preconditioned Jacobi GMRES(m) solve of
    `iters` steps: per step with kp1 = k + 1 basis vectors (k = step mod m)
    the SpMV in the basis type (x gathered through D^-1: + N s_b) and the
    orthogonalisation -- staged CGS2: three passes reading v and the kp1
    vectors, the last writing V_k+1 = (3 (kp1 + 1) + 1) N s_b; MGS: kp1 + 1
    passes reading v, kp1 of them writing it, 2 kp1 basis reads, then the
    normalisation (read v, write V_k+1) = (4 kp1 + 3) N s_b; delayed CGS2:
    two passes reading v and the kp1 vectors, the second writing q_k (k > 0)
    and u_k+1 = (2 (kp1 + 1) + 2) N s_b, and per full cycle one pass of dots
    reading u_m and the m + 1 vectors.  Per cycle end the FP64 correction
    (kp1 = m basis vectors, D^-1, x read and written), the FP64 residual SpMV
    (b read, r written) and basis_0 (read r, write V_0)."""
    sb, n = basis_bytes, nrows
    total = 0
    spmv = spmv_bytes(n, nnz, sb, coding, nblk) + n * sb
    for it in range(iters):
        kp1 = it % m + 1
        if ortho == "cgs2":
            ortho_b = 3 * (kp1 + 1) + 1
        elif ortho == "dcgs2":
            ortho_b = 2 * (kp1 + 1) + (2 if kp1 > 1 else 1)
        else:
            ortho_b = 4 * kp1 + 3
        total += spmv + ortho_b * n * sb
    cycle = (m * sb + 8 + 16) * n + spmv_bytes(n, nnz, 8, coding, nblk) + 16 * n + (8 + sb) * n
    if ortho == "dcgs2":
        total += restarts * (m + 2) * n * sb
    return total + (restarts + 1) * cycle


def pcg_iter_bytes(nrows, nnz, val_bytes, coding=0, nblk=0, kind="fp64"):
    """Algorithmic bytes of one Jacobi-PCG iteration beyond the SpMV's own
    (B_spmv: matrix data, p read once, w written once).
    * "fp64": update (read x, p, r, w, D^-1; write x, r) + direction (read p,
      r, D^-1; write p) = 11 N s_v.
    * "reliable" (mixed): residual update (read r, w, D^-1; write r) +
      direction with the solution step (read p, r, D^-1, x; write p, x) =
      10 N s_v."""
    extra = {"fp64": 11, "reliable": 10}[kind]
    return spmv_bytes(nrows, nnz, val_bytes, coding, nblk) + extra * nrows * val_bytes


def fvm_apply_bytes(n, val_bytes):
    """Algorithmic bytes of one matrix-free finite-volume apply on an n^3 mesh
    with face-coefficient fields: u read once, v written once, and each of
    the three face-transmissibility arrays read once (n^2 (n+1) faces per
    axis)."""
    return val_bytes * (2 * n ** 3 + 3 * n * n * (n + 1))


def _traffic_from_profiles(kernel_key):
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text()).get(kernel_key)
        except Exception:
            return None
    return None


def bench_config(wl, nrows, nnz, ws):
    """The `config` of both arms' lines (the same dict, so that the two
    lines are comparable key for key)."""
    what = (f"{wl} variable-coefficient diffusion, log-normal sigma=1, harmonic faces"
            if wl.startswith("diffusion3d") else wl)
    return {"workload": f"{what}, Jacobi PCG rtol 1e-8",
            "rows": nrows, "nnz": nnz, "parallelism": "replicas" if ws > 1 else "single",
            "l2": "inputs larger than L2 (matrix 1.7 GB), no flush"}


def host_description():
    """The host the CPU legs ran on: logical CPUs and the CPU model."""
    model = None
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                             text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                model = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if model is None:
        try:
            for ln in Path("/proc/cpuinfo").read_text().splitlines():
                if ln.lower().startswith("model name"):
                    model = ln.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    import platform
    return {"nproc": os.cpu_count(), "cpu_model": model, "machine": platform.machine()}


def reference_iters(workload):
    p = ROOT / "tests" / "golden" / "full_size.json"
    if p.exists():
        d = json.loads(p.read_text())
        c = d.get(workload, {}).get("cg")
        if c:
            return int(c["iters"])
    return None


# ------------------------------------------------------------ CPU side --

def _ref_driver():
    p = ROOT / "oracle" / "_ref" / "ref_driver"
    return p if p.exists() else None


def reference_timeline(A, b, maxiter, rtol=1e-8):
    """Run the reference's serial Jacobi-PCG on (A, b) once, from a zero
    guess, with a wall-clock time stamp at every iteration (taken in its
    diagnostic, which the reference's CG calls once per iteration).

    Returns (kind, stamps, total, status, iters): stamps[i] = seconds from the
    start of the solver call to the end of iteration i + 1, total = wall time
    of the whole call.  kind "reference": the reference's own templates
    (oracle/_ref/ref_driver, compiled from its headers); kind "port": the
    oracle restatement, pinned bit-exact to them, where that build is
    absent."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle as O
    drv = _ref_driver()
    if drv is not None:
        import tempfile
        with tempfile.TemporaryDirectory() as td:
            fin, fout, ftim = (os.path.join(td, f) for f in ("in.bin", "out.bin", "t.bin"))
            O.write_problem(fin, A, b, np.zeros(A.nrows))
            env = dict(os.environ, REF_DRIVER_TIMES=ftim)
            subprocess.run([str(drv), fin, fout, "cg", str(int(maxiter)), repr(float(rtol)), "1",
                            "jacobi"], check=True, env=env, stdout=subprocess.PIPE,
                           stderr=subprocess.PIPE)
            raw = open(ftim, "rb").read()
            head = np.fromfile(fout, np.int32, 3)
        ns = int(np.frombuffer(raw, np.int64, 1, 0)[0])
        stamps = np.frombuffer(raw, np.float64, ns, 8).copy()
        total = float(np.frombuffer(raw, np.float64, 1, 8 + 8 * ns)[0])
        return "reference", stamps, total, O.STATUS[int(head[0])], int(head[1])
    stamps = []
    t0 = time.perf_counter()

    def stamp(x, res):
        stamps.append(time.perf_counter() - t0)
        return False
    r = O.solve("cg", A, b, maxiter=int(maxiter), rtol=rtol, diag=stamp)
    total = time.perf_counter() - t0
    return "port", np.array(stamps), total, r.status, r.iters


def cpu_sample(A, b, seconds_target=15.0, max_iters=60):
    """Time a bounded number of iterations of the reference's serial PCG on
    the workload (the reference driver when built, else the oracle port);
    returns (seconds per iteration, iterations timed, kind)."""
    kind, st, total, _, _ = reference_timeline(A, b, 2, rtol=1e-30)
    probe = float(st[-1] - st[0]) if len(st) > 1 else total
    iters = int(max(3, min(max_iters, seconds_target / max(probe, 1e-6))))
    kind, st, total, _, _ = reference_timeline(A, b, iters, rtol=1e-30)
    # per iteration: from the end of the first iteration to the end of the
    # last (the set-up before the first is not part of an iteration)
    return float(st[-1] - st[0]) / max(1, len(st) - 1), len(st) - 1, kind


# ------------------------------------------------------------ GPU side --

def spmv_events_ms(fs, ctx, dA, n, dtype, reps=20):
    """Average duration of one CSR SpMV launch (CUDA events on the library's
    stream around `reps` back-to-back launches, after 3 warm-up launches)."""
    xv = fs.Vector(ctx, n, dtype)
    yv = fs.Vector(ctx, n, dtype)
    xv.set_random(5)
    for _ in range(3):
        dA.apply(xv, yv)
    ctx.sync()
    ctx.record(2)
    for _ in range(reps):
        dA.apply(xv, yv)
    ctx.record(3)
    return ctx.elapsed_ms(2, 3) / reps


def run_spmv_only(args):
    """`--mode spmv`: the SpMV kernel alone on the workload, FP64 then FP32
    (`--steps` timed launches each after `--warmup` ones); the command that
    the ncu summaries of the SpMV kernel are captured from."""
    import flecsolve_gb300 as fs
    from flecsolve_gb300 import problems as P
    A, _ = P.workload(args.workload)
    n, nnz = A.nrows, A.nnz
    ctx = fs.Context(0)
    dA = fs.CSR(ctx, A)
    peak, peak_kind = _peaks()
    best = dA.index_coding()
    out = {"mode": "spmv", "workload": args.workload, "rows": n, "nnz": nnz,
           "index_coding": CODING_NAMES[best]}
    for req in (3, 2, 1, 0):
        # format 3 on a grid stencil with asymmetric values is the general
        # grid storage (4)
        coding = dA.index_coding(req)
        if coding != req and not (req == 3 and coding == 4):
            continue
        for dt, vb in (("f64", 8), ("f32", 4)):
            ms = spmv_events_ms(fs, ctx, dA, n, dt, reps=max(1, args.steps))
            nbytes = spmv_bytes(n, nnz, vb, coding, dA.nblk())
            gbs = nbytes / (ms * 1e-3) / 1e9
            out[dt + "_" + CODING_NAMES[coding]] = {
                "ms": ms, "gbs": gbs, "frac": gbs / peak, "peak": peak,
                "peak_source": f"hbm_gbs of {peak_kind}", "algorithmic_bytes": nbytes}
    if best == 0:
        # no row patterns: the column-id schedules, one thread per row against
        # 4 / 8 / 16 / 32 lanes per row, and the autotuner's choice
        for dt, vb in (("f64", 8), ("f32", 4)):
            npdt = np.float64 if dt == "f64" else np.float32
            nbytes = spmv_bytes(n, nnz, vb, 0, dA.nblk())
            sched = {}
            for lanes in (0, 4, 8, 16, 32, 1):
                dA.set_lanes(lanes, npdt)
                ms = spmv_events_ms(fs, ctx, dA, n, dt, reps=max(1, args.steps))
                name = {0: "row_per_thread", 1: "binned_by_length"}.get(lanes, f"lanes_{lanes}")
                sched[name] = {
                    "ms": ms, "frac": nbytes / (ms * 1e-3) / 1e9 / peak}
            dA.set_lanes(-1, npdt)
            tuned = dA.tune(npdt)
            ms = spmv_events_ms(fs, ctx, dA, n, dt, reps=max(1, args.steps))
            gbs = nbytes / (ms * 1e-3) / 1e9
            out[dt + "_colids_schedules"] = {
                "tuned_lanes": tuned, "ms": ms, "gbs": gbs, "frac": gbs / peak, "peak": peak,
                "peak_source": f"hbm_gbs of {peak_kind}", "algorithmic_bytes": nbytes,
                "rows_nnz_mean": nnz / n, "rows_nnz_max": int(np.diff(A.rowptr).max()),
                "schedules": sched}
    dA.index_coding(min(best, 3))
    return out


def _timed_solve(ctx, slv, vb, vx):
    """One warm solve, then one timed with CUDA events on the library stream."""
    slv(vb, vx)
    ctx.sync()
    ctx.record(6)
    info = slv(vb, vx)
    ctx.record(7)
    return ctx.elapsed_ms(6, 7) * 1e-3, info


def _relres(S, b, x):
    return float(np.linalg.norm(b - S @ x) / np.linalg.norm(b))


def run_suite(args):
    """`--mode suite`: the secondary configurations, one solve each after a
    warm-up (CUDA events), with iteration counts and true FP64 residuals:
    2-D Poisson 128^2 (CG, BiCGSTAB, GMRES(30)); convection-diffusion 192^3
    (BiCGSTAB and GMRES(30), FP64 and mixed); 512 independent 2-D diffusion
    systems in one batched launch against the same solver run system by
    system on a sample; block CG on 16 right-hand sides of the 128^3
    Laplacian against 16 separate solves; the diffusion3d-256 problem as the
    matrix-free finite-volume operator (applies and PCG); NKA with a CG
    preconditioner at 128^3; BDF2 heat at 128^3 with the device time operator;
    the adjoint gradient of
    ||x - x_target||^2 at 128^3 and backward-Euler heat 64^3 x 200 steps
    differentiated with checkpoints every 20."""
    import flecsolve_gb300 as fs
    from flecsolve_gb300 import adjoint as ad
    from flecsolve_gb300 import problems as P
    ctx = fs.Context(0)
    out = {"mode": "suite"}
    only = set(args.suite.split(",")) if args.suite else None

    def want(k):
        return only is None or k in only

    def asked(k):
        # profiling parts: only when named
        return only is not None and k in only

    def krylov(tag, A, b, cases):
        dA = fs.CSR(ctx, A)
        vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
        S = A.to_scipy()
        res = {"rows": A.nrows, "nnz": A.nnz}
        for name, ns, kw in cases:
            slv = ns.solver(ns.settings(maxiter=30000, rtol=1e-8, **kw))(dA, fs.op.jacobi)
            s, info = _timed_solve(ctx, slv, vb, vx)
            res[name] = {"s": s, "iters": info.iters, "restarts": info.restarts,
                         "status": info.status, "true_relres": _relres(S, b, vx.numpy())}
            if name.startswith("gmres") and "max_krylov_dim" in kw:
                # bandwidth bound of the whole solve (algorithmic bytes / HBM peak)
                mixed = "mixed" in name
                ortho = kw.get("ortho", "dcgs2" if mixed else "mgs")
                nbytes = gmres_solve_bytes(A.nrows, A.nnz, dA.index_coding(), dA.nblk(), info.iters,
                                           info.restarts, kw["max_krylov_dim"], ortho,
                                           4 if mixed else 8)
                peak, peak_kind = _peaks()
                res[name]["roofline"] = {
                    "algorithmic_bytes": nbytes, "achieved_gbs": nbytes / s / 1e9,
                    "bound_s": nbytes / (peak * 1e9), "frac": nbytes / (peak * 1e9) / s,
                    "peak_source": f"hbm_gbs of {peak_kind}", "ortho": ortho}
        out[tag] = res

    g30 = dict(max_krylov_dim=30, restart=True)
    if want("poisson2d"):
        A, b = P.workload("poisson2d-128")
        krylov("poisson2d-128", A, b, [("cg", fs.cg, {}), ("bicgstab", fs.bicgstab, {}),
                                       ("gmres30", fs.gmres, g30)])
    if want("convdiff3d"):
        A, b = P.workload("convdiff3d-192")
        krylov("convdiff3d-192", A, b, [
            ("bicgstab", fs.bicgstab, {}), ("bicgstab_mixed", fs.mixed_bicgstab, {}),
            ("gmres30_mgs", fs.gmres, dict(g30, ortho="mgs")),
            ("gmres30_cgs2", fs.gmres, dict(g30, ortho="cgs2")),
            ("gmres30_dcgs2", fs.gmres, dict(g30, ortho="dcgs2")),
            ("gmres30_mixed", fs.mixed_gmres, g30),
            ("gmres30_mixed_cgs2", fs.mixed_gmres, dict(g30, ortho="cgs2"))])
        ref = json.loads((ROOT / "tests" / "golden" / "full_size.json").read_text()).get("convdiff3d-192", {})
        out["convdiff3d-192"]["reference_iters"] = {k: v["iters"] for k, v in ref.items()}
    if want("batched"):
        A, off, b, sides = P.batch_diffusion2d()
        dA = fs.CSR(ctx, A)
        vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
        fs.batch_cg(dA, off, vb, vx, maxiter=20000, rtol=1e-8)  # autotune + warm
        cl, th, nbig = fs.batch_schedule(dA, off)
        ctx.sync()
        ctx.record(6)
        infos = fs.batch_cg(dA, off, vb, vx, maxiter=20000, rtol=1e-8)
        ctx.record(7)
        t = ctx.elapsed_ms(6, 7) * 1e-3
        x = vx.numpy()
        S = A.to_scipy()
        rr = max(_relres(S[off[k]:off[k + 1]], b[off[k]:off[k + 1]], x) for k in range(len(infos)))
        its = [i.iters for i in infos]
        # the same solver on every system separately (the single-system mixed
        # CG, one timed solve each after a warm-up)
        seq = 0.0
        for k in range(len(infos)):
            lo, hi = off[k], off[k + 1]
            Ak = P.CSR(int(hi - lo), int(hi - lo), A.rowptr[lo:hi + 1] - A.rowptr[lo],
                       A.col[A.rowptr[lo]:A.rowptr[hi]] - lo, A.val[A.rowptr[lo]:A.rowptr[hi]])
            slv = fs.mixed_cg.solver(fs.mixed_cg.settings(maxiter=20000, rtol=1e-8))(
                fs.CSR(ctx, Ak), fs.op.jacobi)
            seq += _timed_solve(ctx, slv, fs.Vector(ctx, b[lo:hi]), fs.Vector(ctx, int(hi - lo)))[0]
        # algorithmic bytes: per row and FP32 iteration of the persistent
        # kernel, the SpMV (grid-stencil storage: the diagonal and two upper
        # diagonals; column ids: value + column id per nonzero and the row
        # offset; p read once, A p written), the update (x32 and r read and
        # written, A p and D^-1 read) and the direction (p read and written,
        # D^-1 and r read); the FP64 head iterations and replacements are
        # counted as FP32 ones (a lower bound)
        fmt = fs.batch_format(dA, off)
        rows_it = sum(int(off[k + 1] - off[k]) * its[k] for k in range(len(infos)))
        nnz_row = A.nnz / A.nrows
        b_row_it = (12 if fmt == "grid" else nnz_row * 8 + 4) + 4 + 4 + 24 + 16
        gbs = rows_it * b_row_it / t / 1e9
        peak, peak_kind = _peaks()
        out["batch512-diffusion2d"] = {
            "systems": len(infos), "rows": A.nrows, "nnz": A.nnz, "s": t, "cluster": cl,
            "threads": th, "systems_owning_a_cluster": nbig, "storage": fmt,
            "all_converged": all(i.status == "converged_rtol" for i in infos),
            "max_true_relres": rr, "iters_min": min(its), "iters_max": max(its),
            "iters_sum": int(sum(its)), "row_iterations": rows_it,
            "roofline": {"bytes_per_row_iteration": b_row_it,
                         "algorithmic_bytes": rows_it * b_row_it, "achieved_gbs": gbs,
                         "peak": peak, "frac": gbs / peak, "peak_source": f"hbm_gbs of {peak_kind}"},
            "one_by_one_s": seq,
            "one_by_one": "all 512 systems, single-system mixed CG, one timed solve each"}
    if want("cg-variants"):
        # the CG loops on the headline workload: FP64 (three kernels, two
        # reductions per iteration), the single-reduction FP64 variant (two
        # kernels, one reduction), mixed with and without the FP64 head
        A, b = P.workload("diffusion3d-256")
        dA = fs.CSR(ctx, A)
        vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
        S = A.to_scipy()
        res = {"rows": A.nrows}
        for name, ns, kw in (("cg_fp64", fs.cg, {}), ("cg_fp64_single_reduction", fs.pipelined_cg, {}),
                             ("cg_mixed_fp64_head_3e-3", fs.mixed_cg, {"fp64_head": 3e-3}),
                             ("cg_mixed_fp32_from_start", fs.mixed_cg, {"fp64_head": 0.0})):
            slv = ns.solver(ns.settings(maxiter=20000, rtol=1e-8, **kw))(dA, fs.op.jacobi)
            sec, info = _timed_solve(ctx, slv, vb, vx)
            res[name] = {"s": sec, "iters": info.iters, "status": info.status,
                         "s_per_iteration": sec / max(info.iters, 1),
                         "true_relres": _relres(S, b, vx.numpy())}
        out["cg-variants-diffusion3d-256"] = res
    for part, ortho in (("gmres-profile", "auto"), ("gmres-profile-cgs2", "cgs2")):
        if not asked(part):
            continue
        # profiling: two restart cycles (60 steps) of the mixed GMRES(30) on
        # the 192^3 convection-diffusion system (auto: the delayed CGS2)
        A, b = P.workload("convdiff3d-192")
        dA = fs.CSR(ctx, A)
        vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
        slv = fs.mixed_gmres.solver(fs.mixed_gmres.settings(maxiter=60, rtol=1e-8, max_krylov_dim=30,
                                                            restart=True, ortho=ortho))(dA, fs.op.jacobi)
        info = slv(vb, vx)
        ctx.sync()
        out[f"convdiff3d-192-mixed-gmres-60-{ortho}"] = {"iters": info.iters, "status": info.status}
    if asked("bicgstab-profile"):
        # profiling: 40 iterations of the mixed BiCGSTAB on the 192^3
        # convection-diffusion system
        A, b = P.workload("convdiff3d-192")
        dA = fs.CSR(ctx, A)
        vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
        slv = fs.mixed_bicgstab.solver(fs.mixed_bicgstab.settings(maxiter=40, rtol=1e-8))(dA, fs.op.jacobi)
        info = slv(vb, vx)
        ctx.sync()
        out["convdiff3d-192-mixed-bicgstab-40"] = {"iters": info.iters, "status": info.status}
    if asked("batched-profile"):
        # profiling: 128 systems of side 96..200 in one launch (about 0.3 GB
        # of vectors and coefficients, more than L2), cluster 2 x 256 threads
        # (no autotuning launches)
        A, off, b, _ = P.batch_diffusion2d(nsys=128, side_lo=96, side_hi=200)
        dA = fs.CSR(ctx, A)
        vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, A.nrows)
        infos = fs.batch_cg(dA, off, vb, vx, maxiter=20000, rtol=1e-8, cluster=2, threads=256)
        ctx.sync()
        out["batch128-diffusion2d-96-200"] = {
            "rows": A.nrows, "nnz": A.nnz, "storage": fs.batch_format(dA, off),
            "iters_sum": int(sum(i.iters for i in infos)),
            "row_iterations": sum(int(off[k + 1] - off[k]) * infos[k].iters for k in range(len(infos)))}
    if want("blockcg-mixed"):
        # the mixed block solve alone (profiling): 16 right-hand sides of the
        # 96^3 Laplacian, one warm-up and one timed solve
        A, _ = P.workload("laplace3d-96")
        n = A.nrows
        B = np.stack([P.uniform(6 + j, n) for j in range(16)], axis=1)
        dA = fs.CSR(ctx, A)
        vB, vX = fs.Vector(ctx, B.ravel()), fs.Vector(ctx, n * 16)
        fs.block_cg(dA, vB, vX, 16, maxiter=5000, rtol=1e-8, mixed=True)
        ctx.sync()
        ctx.record(6)
        infos = fs.block_cg(dA, vB, vX, 16, maxiter=5000, rtol=1e-8, mixed=True)
        ctx.record(7)
        out["laplace3d-96x16-mixed"] = {"s": ctx.elapsed_ms(6, 7) * 1e-3,
                                        "block_iters": infos[0].restarts}
    if want("blockcg"):
        A, _ = P.workload("laplace3d-128")
        n = A.nrows
        B = np.stack([P.uniform(6 + j, n) for j in range(16)], axis=1)
        dA = fs.CSR(ctx, A)
        S = A.to_scipy()
        res = {"rows": n, "nnz": A.nnz, "rhs": 16}
        vB, vX = fs.Vector(ctx, B.ravel()), fs.Vector(ctx, n * 16)
        fs.block_cg(dA, vB, vX, 16, maxiter=5000, rtol=1e-8)
        ctx.sync()
        ctx.record(6)
        infos = fs.block_cg(dA, vB, vX, 16, maxiter=5000, rtol=1e-8)
        ctx.record(7)
        X = vX.numpy().reshape(n, 16)
        res["block_cg_fp64"] = {"s": ctx.elapsed_ms(6, 7) * 1e-3, "block_iters": infos[0].restarts,
                                "max_true_relres": max(_relres(S, B[:, j], X[:, j]) for j in range(16))}
        fs.block_cg(dA, vB, vX, 16, maxiter=5000, rtol=1e-8, mixed=True)
        ctx.sync()
        ctx.record(6)
        infos = fs.block_cg(dA, vB, vX, 16, maxiter=5000, rtol=1e-8, mixed=True)
        ctx.record(7)
        X = vX.numpy().reshape(n, 16)
        res["block_cg_mixed"] = {"s": ctx.elapsed_ms(6, 7) * 1e-3, "block_iters": infos[0].restarts,
                                 "all_converged": all(i.status == "converged_rtol" for i in infos),
                                 "max_true_relres": max(_relres(S, B[:, j], X[:, j]) for j in range(16))}
        for name, ns in (("16x_pcg_fp64", fs.cg), ("16x_pcg_mixed", fs.mixed_cg)):
            vb, vx = fs.Vector(ctx, n), fs.Vector(ctx, n)
            slv = ns.solver(ns.settings(maxiter=5000, rtol=1e-8))(dA, fs.op.jacobi)
            tot, its = 0.0, []
            for j in range(16):
                vb.upload(B[:, j])
                s, info = _timed_solve(ctx, slv, vb, vx)
                tot += s
                its.append(info.iters)
            res[name] = {"s": tot, "iters_max": max(its), "iters_sum": sum(its)}
        out["laplace3d-128x16"] = res
    if want("fvm") or want("fvm-apply"):
        # the matrix-free finite-volume operator on the diffusion3d-256
        # problem: the generator's face coefficients as face fields, Dirichlet
        # 0 on every face and dA/dx = 1 (box [0, n+1]^3) give the same
        # operator as the assembled matrix
        from flecsolve_gb300 import physics as ph
        n = 256
        A, b = P.workload(f"diffusion3d-{n}")
        N = A.nrows
        mesh = ph.fvm_mesh(ctx, (n, n, n), [(0.0, float(n + 1))] * 3)
        fields = mesh.face_fields(P.faces_to_fields(n, P.faces_lognormal(3, n, seed=2)))
        Amf = ph.op_expr(*[ph.bc(ph.dirichlet(0.0), f // 2, f % 2) for f in range(6)],
                         ph.diffusion(mesh, None, fields, 1.0, 0.0)).matrix_free()
        del fields
        peak, peak_kind = _peaks()
        res = {"rows": N, "problem": "diffusion3d-256 as a matrix-free operator (face fields, Dirichlet 0)"}
        for dt, vbytes in (("f64", 8), ("f32", 4)):
            ms = spmv_events_ms(fs, ctx, Amf, N, dt, reps=20)
            nbytes = fvm_apply_bytes(n, vbytes)
            gbs = nbytes / (ms * 1e-3) / 1e9
            res["apply_" + dt] = {"ms": ms, "gbs": gbs, "frac": gbs / peak, "peak": peak,
                                  "peak_source": f"hbm_gbs of {peak_kind}", "algorithmic_bytes": nbytes}
        S = A.to_scipy()
        x = P.uniform(5, N)
        y = fs.Vector(ctx, N)
        Amf.apply(fs.Vector(ctx, x), y)
        ref = S @ x
        res["max_rel_diff_vs_matrix"] = float(np.abs(y.numpy() - ref).max() / np.abs(ref).max())
        if want("fvm"):
            vb, vx = fs.Vector(ctx, b), fs.Vector(ctx, N)
            for name, ns in (("pcg_fp64", fs.cg), ("pcg_mixed", fs.mixed_cg)):
                slv = ns.solver(ns.settings(maxiter=20000, rtol=1e-8))(Amf, fs.op.jacobi)
                s, info = _timed_solve(ctx, slv, vb, vx)
                res[name] = {"s": s, "iters": info.iters, "status": info.status,
                             "true_relres": _relres(S, b, vx.numpy())}
        out["fvm-diffusion3d-256"] = res
    if want("nka"):
        # NKA with a CG preconditioner set up as solvers/test/nka.cc does (b = 1,
        # x0 = 3, nka.cfg: max_dim 5, angle 0.2) on the 128^3 log-normal
        # diffusion operator, with the preconditioner's CG at 100 iterations
        # (the test's 11 suit its 64^2 Poisson problem) and atol 1e-3
        # (||b|| = 1448)
        A, _ = P.workload("diffusion3d-128")
        dA = fs.CSR(ctx, A)
        vb = fs.Vector(ctx, np.ones(A.nrows))
        pre = fs.cg.solver(fs.cg.settings(maxiter=100, rtol=1e-9, atol=1e-9, use_zero_guess=True),
                           fs.cg.make_work(vb))(dA)
        s_nka = fs.nka.settings(maxiter=500, atol=1e-3, max_dim=5, angle_tol=0.2, use_zero_guess=False)
        res = {"rows": A.nrows, "nnz": A.nnz}
        for rep in range(2):  # the first solve warms up the preconditioner's graphs
            vx = fs.Vector(ctx, np.full(A.nrows, 3.0))
            slv = fs.nka.solver(s_nka, fs.nka.make_work(vb, 10))(dA, pre)
            ctx.sync()
            t0 = time.perf_counter()
            info = slv(vb, vx)
            ctx.sync()
            t = time.perf_counter() - t0
        res["nka_cg100"] = {"s": t, "iters": info.iters, "status": info.status,
                           "s_per_iteration": t / max(info.iters, 1),
                           "true_res": float(np.linalg.norm(np.ones(A.nrows) - A.to_scipy() @ vx.numpy()))}
        out["nka-diffusion3d-128"] = res
    if want("bdf"):
        # BDF2 with the truncation-error controller on the heat equation
        # u' = -A u (A the 128^3 log-normal diffusion operator, u0 U[0,1]):
        # the time operator I + gamma A on the device, mixed-precision Jacobi
        # CG as the time solver; the host controller's share of the wall time
        from flecsolve_gb300.time_integrator import bdf
        A, _ = P.workload("diffusion3d-128")
        J = fs.CSR(ctx, P.CSR(A.nrows, A.ncols, A.rowptr, A.col, -A.val))
        st = bdf.settings(**{"initial-time": 0.0, "final-time": 2.0, "initial-dt": 1e-3, "max-dt": 0.5,
                             "max-steps": 10000, "timestep-selection-strategy": "truncation-error",
                             "integrator": "BDF2", "starting-integrator": "CN", "predictor": "leapfrog",
                             "trunc-error-rtol": 1e-4, "trunc-error-atol": 1e-6,
                             "time-error-scaling": "fixed-resolution", "time-trunc-error-norm": "inf"})
        res = {"rows": A.nrows, "problem": "u' = -A u, diffusion3d-128, t in [0, 2]"}
        for rep in range(2):  # the first run warms up the solver's graphs
            ti = bdf.linear(st, J, fs.mixed_cg.settings(maxiter=20000, rtol=1e-8, use_zero_guess=False),
                            P=fs.op.jacobi)
            x, xn = fs.Vector(ctx, P.uniform(17, A.nrows, 0.0, 1.0)), fs.Vector(ctx, A.nrows)
            ctx.sync()
            t0 = time.perf_counter()
            dt, first, attempts, iters = ti.get_current_dt(), True, 0, 0
            while ti.get_current_time() < ti.get_final_time():
                ti.advance(dt, first, x, xn)
                iters += ti.last_solver_iters()
                attempts += 1
                good = ti.check_solution()
                if good:
                    ti.update()
                    x, xn = xn, x
                    first = False
                dt = ti.get_next_dt(good)
            ctx.sync()
            t = time.perf_counter() - t0
        res["bdf2_mixed_cg"] = {"s": t, "steps": ti.get_current_step(), "rejects": ti.num_step_rejects(),
                                "attempts": attempts, "krylov_iters": iters,
                                "s_per_attempt": t / max(attempts, 1)}
        # the same number of Krylov iterations as plain solves: the time
        # solver's share of the wall time
        vb, vx = fs.Vector(ctx, P.uniform(3, A.nrows)), fs.Vector(ctx, A.nrows)
        Tm = P.CSR(A.nrows, A.ncols, A.rowptr, A.col, A.val * 0.01)
        Tm.val[Tm.col == np.repeat(np.arange(A.nrows), np.diff(A.rowptr))] += 1.0
        slv = fs.mixed_cg.solver(fs.mixed_cg.settings(maxiter=20000, rtol=1e-8))(fs.CSR(ctx, Tm), fs.op.jacobi)
        s1, info1 = _timed_solve(ctx, slv, vb, vx)
        res["time_operator_solve_probe"] = {"s": s1, "iters": info1.iters,
                                            "s_per_krylov_iter": s1 / max(info1.iters, 1)}
        out["bdf-heat-diffusion3d-128"] = res
    if want("adjoint"):
        n = 128
        system = ad.DiffusionSolve(ctx, 3, n, rtol=1e-8)
        c = P.faces_lognormal(3, n, seed=2)
        b = P.uniform(3, n ** 3)
        system.set_faces(P.faces_lognormal(3, n, seed=7))
        vb, xt = fs.Vector(ctx, b), fs.Vector(ctx, n ** 3)
        system.solve(vb, xt)
        t_h = xt.numpy()
        x = fs.Vector(ctx, n ** 3)
        system.set_faces(c)
        g = fs.Vector(ctx, n ** 3)
        for rep in range(2):
            ctx.sync()
            ctx.record(6)
            system.solve(vb, x)                     # forward
            g.linear_sum(2.0, x, -2.0, xt)          # dL/dx
            system.adjoint(g, x)                    # A^T lam = dL/dx, dL/dc
            ctx.record(7)
        out["adjoint-diffusion3d-128"] = {
            "s_forward_plus_gradient": ctx.elapsed_ms(6, 7) * 1e-3,
            "gradient_entries": system.nfaces + n ** 3}
        n, dt, steps = 64, 1e-3, 200
        heat = ad.DiffusionSolve(ctx, 3, n, rtol=1e-8, scale=dt, shift=1.0)
        u0 = P.uniform(9, n ** 3)
        heat.set_faces(P.faces_lognormal(3, n, seed=7))
        target = ad.heat_forward(heat, u0, steps)[0].numpy()
        cf = P.faces_lognormal(3, n, seed=2)
        t0 = time.perf_counter()
        heat.set_faces(cf)
        ad.heat_forward(heat, u0, steps)
        ctx.sync()
        t_fwd = time.perf_counter() - t0
        t0 = time.perf_counter()
        ad.heat_loss_and_grad(heat, cf, u0, target, steps, checkpoint=20)
        ctx.sync()
        out["heat-be-64x200"] = {"s_forward": t_fwd, "s_loss_and_gradient": time.perf_counter() - t0,
                                 "checkpoint_every": 20, "states_held": 20 + 1 + steps // 20}
    return out


def run_ours(args, ws, rank, local):
    import flecsolve_gb300 as fs
    from flecsolve_gb300 import problems as P

    wl = args.workload
    t0 = time.perf_counter()
    A, b = P.workload(wl)
    gen_s = time.perf_counter() - t0
    n, nnz = A.nrows, A.nnz
    ctx = fs.Context(local)
    dA = fs.CSR(ctx, A)
    vb = fs.Vector(ctx, b)
    vx = fs.Vector(ctx, n)
    s64 = fs.cg.settings(maxiter=args.maxiter, rtol=1e-8, use_zero_guess=True)
    smx = fs.mixed_cg.settings(maxiter=args.maxiter, rtol=1e-8, use_zero_guess=True,
                               inner_rtol=args.inner_rtol, refine=args.refine,
                               fp64_head=args.fp64_head)
    smx0 = fs.mixed_cg.settings(maxiter=args.maxiter, rtol=1e-8, use_zero_guess=True,
                                inner_rtol=args.inner_rtol, refine=args.refine, fp64_head=0.0)
    cg64 = fs.cg.solver(s64, fs.cg.make_work(vb))(fs.op.ref(dA), fs.op.jacobi)
    cgmx = fs.mixed_cg.solver(smx, fs.mixed_cg.make_work(vb))(fs.op.ref(dA), fs.op.jacobi)
    cgmx0 = fs.mixed_cg.solver(smx0, fs.mixed_cg.make_work(vb))(fs.op.ref(dA), fs.op.jacobi)

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    def timed(slv, K, W, tag):
        for _ in range(W):
            info = slv(vb, vx)
        barrier()
        ctx.sync()
        l0 = ctx.launches
        ctx.record(0)
        infos = []
        for _ in range(K):
            infos.append(slv(vb, vx))
        ctx.record(1)
        ms = ctx.elapsed_ms(0, 1)
        ctx.sync()
        barrier()
        return ms / K, infos[-1], ctx.launches - l0

    with ClockSampler(local) as clk:
        ms_mx, info_mx, launches_mx = timed(cgmx, args.steps, args.warmup, "mixed")
    clocks = clk.summary()
    x_mx = vx.numpy()
    ms_64, info_64, launches_64 = timed(cg64, args.steps, max(1, args.warmup // 3), "fp64")
    x_64 = vx.numpy()
    ms_mx0, info_mx0, _ = timed(cgmx0, args.steps, max(1, args.warmup // 3), "mixed-fp32-start")
    x_mx0 = vx.numpy()
    # a tight FP64 solve (rtol 1e-12, untimed): the forward error of each result
    tight = fs.cg.solver(fs.cg.settings(maxiter=args.maxiter, rtol=1e-12, use_zero_guess=True),
                         fs.cg.make_work(vb))(fs.op.ref(dA), fs.op.jacobi)
    info_t = tight(vb, vx)
    x_t = vx.numpy()

    # max over ranks of the per-step time
    ms_mx, ms_64, ms_mx0 = max_over_ranks([ms_mx, ms_64, ms_mx0], ws)

    # SpMV kernel alone (the dominant kernel), CUDA events on the same stream
    spmv64_ms = spmv_events_ms(fs, ctx, dA, n, "f64")
    spmv32_ms = spmv_events_ms(fs, ctx, dA, n, "f32")
    peak, peak_kind = _peaks()
    coding = dA.index_coding()
    cname = CODING_NAMES[coding]
    b64 = spmv_bytes(n, nnz, 8, coding, dA.nblk())
    b32 = spmv_bytes(n, nnz, 4, coding, dA.nblk())
    gbs64 = b64 / (spmv64_ms * 1e-3) / 1e9
    gbs32 = b32 / (spmv32_ms * 1e-3) / 1e9
    # whole mixed iteration: two kernels when the SpMV stages windows
    it_bytes = pcg_iter_bytes(n, nnz, 4, coding, dA.nblk(), "reliable")
    # the FP32 iteration: from the solve with FP32 recurrences from the start
    it_s = ms_mx0 * 1e-3 / max(1, info_mx0.iters)

    # e2e: through the public API with host buffers
    import torch
    hb = torch.from_numpy(b).pin_memory()
    hx = torch.empty(n, dtype=torch.float64).pin_memory()
    import ctypes as C
    from flecsolve_gb300._lib import lib, check
    L = lib()
    for _ in range(max(1, args.warmup // 3)):
        check(L.fs_vec_upload(vb.h, C.c_void_p(hb.data_ptr()), n), ctx.h)
        cgmx(vb, vx)
        check(L.fs_vec_download(vx.h, C.c_void_p(hx.data_ptr()), n), ctx.h)
    barrier()
    ctx.sync()
    ctx.record(4)
    for _ in range(args.steps):
        check(L.fs_vec_upload(vb.h, C.c_void_p(hb.data_ptr()), n), ctx.h)
        cgmx(vb, vx)
        check(L.fs_vec_download(vx.h, C.c_void_p(hx.data_ptr()), n), ctx.h)
    ctx.record(5)
    e2e_ms = ctx.elapsed_ms(4, 5) / args.steps
    barrier()

    # accuracy of the headline result against the FP64 GPU solve, and the
    # true FP64 relative residual of both
    sys.path.insert(0, str(ROOT / "oracle"))
    S = A.to_scipy()

    def relres(x):
        return float(np.linalg.norm(b - S @ x) / np.linalg.norm(b))

    def rel(x, y):
        return float(np.linalg.norm(x - y) / np.linalg.norm(y))
    relres_mx, relres_64, relres_mx0 = relres(x_mx), relres(x_64), relres(x_mx0)
    err_vs_fp64 = rel(x_mx, x_64)
    # the reference's own solution of this workload at 1024 rows
    vs_ref = None
    fsz = ROOT / "tests" / "golden" / "full_size.json"
    if fsz.exists():
        ref = json.loads(fsz.read_text()).get(wl, {}).get("cg")
        if ref:
            idx = np.asarray(ref["x_sample_index"])
            xs = np.asarray(ref["x_sample"])
            vs_ref = {"fp64_pcg": rel(x_64[idx], xs), "mixed_pcg": rel(x_mx[idx], xs),
                      "reference_iters": ref["iters"],
                      "what": "relative distance to the reference's own solution at 1024 sampled rows"}

    out = {
        "metric": METRIC,
        "value": ms_mx * 1e-3,
        "unit": "s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_mx,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32-inner/f64-refine",
        "data": "synthetic (seeded generator, no dataset)",
        "config": bench_config(wl, n, nnz, ws),
        "fp64_pcg": {"s": ms_64 * 1e-3, "iters": info_64.iters, "status": info_64.status,
                     "true_relres": relres_64, "launches_per_step": launches_64 / args.steps,
                     "forward_err_vs_tight_fp64": rel(x_64, x_t)},
        "mixed_pcg": {"s": ms_mx * 1e-3, "iters": info_mx.iters, "outer": info_mx.restarts,
                      "status": info_mx.status, "true_relres": relres_mx,
                      "rel_err_vs_fp64_gpu": err_vs_fp64,
                      "forward_err_vs_tight_fp64": rel(x_mx, x_t),
                      "fp64_head": args.fp64_head, "refine": args.refine,
                      "inner_rtol": args.inner_rtol or ("library default (0.1)" if args.refine == "reliable" else "library default (1e-4)")},
        "mixed_pcg_fp32_from_start": {
            "s": ms_mx0 * 1e-3, "iters": info_mx0.iters, "status": info_mx0.status,
            "true_relres": relres_mx0, "rel_err_vs_fp64_gpu": rel(x_mx0, x_64),
            "forward_err_vs_tight_fp64": rel(x_mx0, x_t), "speedup_vs_fp64": ms_64 / ms_mx0},
        "tight_fp64_solve": {"rtol": 1e-12, "iters": info_t.iters, "status": info_t.status},
        "vs_reference_solution": vs_ref,
        "speedup_mixed_vs_fp64": ms_64 / ms_mx,
        "spmv_hbm_gbs": {"f64": gbs64, "f32": gbs32, "f64_ms": spmv64_ms, "f32_ms": spmv32_ms},
        "roofline": {"bound": "hbm",
                     "kernel": {3: "spmv_grid_kernel<float> (FP32 CSR SpMV, grid stencil: diagonal + upper diagonals addressed by grid coordinates, 16-byte loads)",
                                2: "spmv_sym_kernel<float> (FP32 CSR SpMV, symmetric storage: diagonal + upper diagonals)",
                                1: "spmv_pat_kernel<float> (FP32 CSR SpMV, row patterns, warp-specialised)",
                                0: "spmv_rb_kernel<float> (FP32 CSR SpMV, int32 column ids)"}[coding],
                     "achieved": gbs32, "peak": peak, "unit": "GB/s", "frac": gbs32 / peak,
                     "peak_source": f"hbm_gbs of {peak_kind}",
                     "algorithmic_bytes_per_launch": b32,
                     "traffic": _traffic_from_profiles(f"spmv_f32_{cname}")},
        "roofline_fp64_spmv": {"achieved": gbs64, "peak": peak, "frac": gbs64 / peak,
                               "algorithmic_bytes_per_launch": b64,
                               "traffic": _traffic_from_profiles(f"spmv_f64_{cname}")},
        "roofline_mixed_iteration": {"bytes_per_iteration": it_bytes, "s_per_iteration": it_s,
                                     "achieved": it_bytes / it_s / 1e9, "peak": peak,
                                     "frac": it_bytes / it_s / 1e9 / peak,
                                     "kernels_per_iteration": 3,
                                     "from": "mixed_pcg_fp32_from_start (every iteration FP32)"},
        "e2e": {"value": e2e_ms * 1e-3, "unit": "s", "h2d_bytes_per_step": 8 * n,
                "d2h_bytes_per_step": 8 * n},
        "gpu_launches": launches_mx,
        "clocks": clocks,
        "setup": {"generate_s": gen_s},
    }
    if rank == 0 and not args.no_cpu:
        per_it, its, kind = cpu_sample(A, b, args.cpu_seconds)
        ref_it = reference_iters(wl) or info_64.iters
        what = ("the reference's serial Jacobi-PCG (its own templates, oracle/_ref/ref_driver)"
                if kind == "reference" else
                "the oracle (the reference's serial PCG restated in C, pinned bit-exact to it)")
        out["cpu_baseline"] = {"value": per_it * ref_it, "unit": "s", "cores": 1, "kind": kind,
                               "projected": True, "host": host_description(),
                               "sample": f"{its} Jacobi-PCG iterations of {wl} timed with {what}: "
                                         f"{per_it:.4f} s/iter x {ref_it} reference iterations "
                                         f"(a projection; `bench.py --impl reference` times the "
                                         f"complete solve)"}
    return out


def run_reference(args, ws, rank, local):
    """One complete solve of the reference's serial Jacobi-PCG, split into
    the W + K steps the contract times (see the module docstring)."""
    from flecsolve_gb300 import problems as P
    wl = args.workload
    A, b = P.workload(wl)
    kind, stamps, total, status, iters = reference_timeline(A, b, args.maxiter)
    nst = len(stamps)
    nsteps = args.warmup + args.steps
    # chunk boundaries over the iterations; chunk c ends at iteration e_c
    ends = [max(1, round((c + 1) * nst / nsteps)) for c in range(nsteps)]
    chunk_s = []
    prev = 0.0
    for e in ends:
        t = float(stamps[e - 1]) if nst else total
        chunk_s.append(t - prev)
        prev = t
    timed = chunk_s[args.warmup:]
    ms_per_step = 1e3 * sum(timed) / max(1, len(timed))
    what = ("the reference's own serial Jacobi-PCG templates (flecsolve/solvers/cg.hh over "
            "vec::seq_vec and mat::csr<double>), compiled from its headers into "
            "oracle/_ref/ref_driver" if kind == "reference" else
            "the oracle (the reference's serial PCG restated in C, pinned bit-exact to it; "
            "the reference build is absent on this host)")
    sample = (f"one complete solve of {wl} to rtol 1e-8 ({iters} iterations, {status}) with "
              f"{what}, one core (the reference's serial path); the {nsteps} steps are "
              f"{nsteps} consecutive chunks of its iterations, the first with the set-up; "
              f"value = the measured wall time of the whole solve")
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": total,
        "unit": "s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded generator, no dataset)",
        "config": bench_config(wl, A.nrows, A.nnz, ws),
        "step": "a chunk of consecutive iterations of one complete solve (value: that solve)",
        "reference_solve": {"s": total, "iters": iters, "status": status,
                            "s_per_iteration": (float(stamps[-1] - stamps[0]) / max(1, nst - 1)
                                                if nst > 1 else None),
                            "chunk_s": chunk_s},
        "cpu_baseline": {"value": total, "unit": "s", "cores": 1, "kind": kind,
                         "projected": False, "host": host_description(), "sample": sample},
        "e2e": {"value": total, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="diffusion3d-256")
    ap.add_argument("--maxiter", type=int, default=20000)
    ap.add_argument("--inner-rtol", dest="inner_rtol", type=float, default=0.0,
                    help="replacement factor (reliable) / inner tolerance (restart); 0 = library default")
    ap.add_argument("--refine", default="reliable", choices=["restart", "reliable"])
    ap.add_argument("--fp64-head", dest="fp64_head", type=float, default=3e-3,
                    help="mixed CG: FP64 iterations until the residual is below this "
                         "fraction of ||b|| (0 = FP32 recurrences from the start)")
    ap.add_argument("--cpu-seconds", dest="cpu_seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", dest="no_cpu", action="store_true")
    ap.add_argument("--mode", default="solve", choices=["solve", "spmv", "suite"],
                    help="spmv: time only the SpMV kernel on the workload (profiling); "
                         "suite: the secondary configurations")
    ap.add_argument("--suite", default="", help="comma list of suite parts (default: all)")
    args = ap.parse_args()
    if args.mode == "spmv":
        print(json.dumps(run_spmv_only(args)))
        return
    if args.mode == "suite":
        print(json.dumps(run_suite(args)))
        return
    ws, rank, local = _dist()
    if ws > 1:
        import torch
        import torch.distributed as dist
        if args.impl == "reference":
            if rank != 0:
                return
        else:
            torch.cuda.set_device(local)
            dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if args.impl == "reference":
        out = run_reference(args, ws, rank, local)
    else:
        out = run_ours(args, ws, rank, local)
    if rank == 0:
        print(json.dumps(out))
    if ws > 1 and args.impl != "reference":
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
