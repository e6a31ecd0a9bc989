"""Benchmark of the QSM hot path on GB300: single-step TGV-QSM inversion.

Workload (one step = one full inversion): 224x224x128 voxels, 1 mm
isotropic, B0 along z, 60-ellipsoid phantom in an ellipsoidal brain mask,
lam = 0.003, alpha = 2, 1000 iterations, tol = 0 (every step runs all 1000
iterations).  Synthetic, seeded (qsm_gb300.synthetic.config2).

Arms (JSON line on rank 0):
  value         mixed-precision fused path (FP32 stencils, monitors summed in
                compensated FP32 per thread and FP64 across threads),
                inputs resident in HBM, voxel-iterations per second over all
                ranks; every step allocates/initialises its solver state and
                runs the 1000 iterations; the ~1 GB working set exceeds L2.
  e2e           the same call through the C ABI with pinned HOST buffers
                (d2f and mask copied in, chi copied out inside the timing).
  fp64_plain    the plain FP64 path (reference loop structure, bit-identical
                to the reference MEX), for the mixed-vs-FP64 ratio; the
                mixed result's relative L2 error is taken against it.
  roofline      the fused kernel: algorithmic bytes per launch (166 B per
                voxel-iteration x the mask voxels of the interior, whose state
                the kernel reads and writes) / average launch time measured
                with CUDA events on the library's stream; peak from
                MEASURED_PEAKS.json; beside it the DRAM bytes an ncu capture
                of this kernel build measured per launch and their fraction.
  cpu_baseline  the CPU oracle (a C restatement of the reference MEX,
                bit-exact with it; OpenMP on all host cores): its FP32 path on
                a bounded iteration sample, and its FP64 path for all 1000
                iterations, whose chi the mixed result is compared against.
  poisson, batch, served, next_rows
                the MG-PCG solve, batched TV, served requests, and the widened
                rows (TV ADMM, PDF, V-SHARP, whole sstgv/lbv wrappers), each
                with its own workload description.

--impl reference times that CPU implementation alone (the reference's MEX
path cannot run on the GPU host: it needs MATLAB, and its sources are not
shipped there), on the same workload and metric.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import struct
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "TGV voxel-iter/s & HBM GB/s, mixed vs FP64 GPU at ≤1e-4 rel err; served p50/p99"
ITERS = 1000
LAM, ALPHA = 0.003, 2.0
ALG_BYTES_FP32 = 166  # algorithmic bytes per voxel-iteration of fused FP32 TGV
# DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum) per launch of the fused
# kernel on the headline workload, from one single-pass ncu capture per kernel build and
# tile (profiles/tgv_224x224x128_launch_list.md).  Keyed by a digest of the kernel's source
# files, so a kernel changed since its capture reports no traffic rather than a stale one.
KERNEL_SOURCES = ("qsm.m_gb300/csrc/pd_tile.cuh", "qsm.m_gb300/csrc/pd_fused.cuh", "qsm.m_gb300/csrc/pd_stream.cu",
                  "qsm.m_gb300/csrc/pd_tma.cuh")
NCU_TRAFFIC_224x224x128 = {  # (digest, tx, ty, z-chunk) -> bytes per launch
    ("2e157d096d22f024", 28, 16, 16): 275.6e6,  # median of 5 launches: read 190.9 MB + write 84.7 MB
}


def kernel_digest() -> str:
    """Digest of the kernel's source files with comments and blank lines
    removed: edits to comments keep it, any code change moves it."""
    import hashlib
    import re

    h = hashlib.sha256()
    for rel in KERNEL_SOURCES:
        with open(os.path.join(ROOT, rel), encoding="utf-8") as fh:
            src = fh.read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        code = "\n".join(ln.rstrip() for ln in src.splitlines() if ln.strip())
        h.update(code.encode())
    return h.hexdigest()[:16]
WORKLOAD = "TGV-QSM 224x224x128, 1 mm isotropic, B0 along z, 1000 iterations, tol 0"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, dist=None, device="cpu") -> float:
    """The largest x over all ranks, returned on every rank (x itself without a
    process group): the step time a multi-replica run reports."""
    if dist is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world_size: int, seconds: float) -> float:
    """Units all replicas processed per second of the slowest replica (weak scaling)."""
    return world_size * units_per_rank / seconds


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        rows = []
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), parts[4:8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, flags in rows for i, f in enumerate(flags) if f.lower() == "active"})
        sm = sorted(r[0] for r in rows)
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows)}


def _case(shape=None):
    import qsm_gb300.synthetic as S

    if shape is None:
        d2f, mask, _ = S.config2(seed=2)
    else:  # reduced volume for profiler captures, same recipe scaled
        semi = tuple(0.42 * n for n in shape)
        d2f, mask, _ = S.tgv_case(shape, 2, n_ell=60, chi=(-0.15, 0.15), noise=0.02,
                                  mask=S.ellipsoid_mask(shape, semi))
    return d2f, mask


def _cpu_model() -> str:
    """Host CPU description for the baseline record (model name when the kernel gives one)."""
    import platform

    name = ""
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if line.lower().startswith(("model name", "cpu model", "hardware")):
                    name = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    if not name:  # Arm kernels list implementer / part codes only; lscpu names the core
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            name = next((ln.split(":", 1)[1].strip() for ln in out.splitlines()
                         if ln.lower().startswith("model name")), "")
        except (OSError, subprocess.SubprocessError):
            pass
    return f"{name or platform.processor() or 'unknown'} ({platform.machine()}, {os.cpu_count()} cores)"


def _port():
    """The CPU oracle (oracle/liborc.so, built here if needed): only the CPU legs use it."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    import port

    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    return port


def _cores() -> int:
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def _tgv_sample(port, d2f, mask, budget_s):
    """A bounded iteration sample of the TGV inversion on the CPU oracle:
    (iterations, seconds), the count sized from two probes so the sample
    takes about budget_s."""
    t = time.perf_counter()
    port.pd_tgv_mex(d2f, mask, [1, 1, 1], LAM, ALPHA, 0.0, 5)
    t5 = time.perf_counter() - t
    t = time.perf_counter()
    port.pd_tgv_mex(d2f, mask, [1, 1, 1], LAM, ALPHA, 0.0, 15)
    t15 = time.perf_counter() - t
    per_iter = max((t15 - t5) / 10, t15 / 15 / 4, 1e-6)  # the difference drops the set-up cost
    iters = int(max(10, min(ITERS, budget_s / per_iter)))
    iters -= iters % 10
    t = time.perf_counter()
    port.pd_tgv_mex(d2f, mask, [1, 1, 1], LAM, ALPHA, 0.0, iters)
    return iters, time.perf_counter() - t


def cpu_baseline(d2f, mask, budget_s=12.0):
    """The CPU oracle (a C restatement of the reference MEX, bit-exact with it;
    OpenMP on every host core) on the headline inversion.  Its FP32 path
    (mx_pdf, the algorithm the fused kernel reproduces bit for bit) on a
    bounded iteration sample is the like-for-like baseline; its FP64 path
    (mx_pdd) runs all 1000 iterations, and that chi is the FP64 oracle the
    mixed result's error is measured against.  Returns (record, chi64)."""
    port = _port()
    n = d2f.size
    d32 = np.asfortranarray(d2f.astype(np.float32))
    it32, s32 = _tgv_sample(port, d32, mask, budget_s)
    t = time.perf_counter()
    chi64 = port.pd_tgv_mex(d2f, mask, [1, 1, 1], LAM, ALPHA, 0.0, ITERS)
    s64 = time.perf_counter() - t
    rec = {"value": n * it32 / s32, "unit": "voxel-iter/s", "cores": _cores(), "kind": "port", "dtype": "f32",
           "seconds": s32, "cpu": _cpu_model(),
           "sample": f"{it32} of the {ITERS} FP32 iterations (mx_pdf) of the same 224x224x128 TGV inversion "
                     "(CPU oracle, OpenMP)",
           "fp64": {"value": n * ITERS / s64, "unit": "voxel-iter/s", "seconds": s64,
                    "sample": f"all {ITERS} FP64 iterations (mx_pdd), the FP64 oracle chi"}}
    return rec, chi64


def _coarsen(G):
    """Next-level mask (coarsen_grid_mex.c:52-125): coarse interior voxel =
    AND of its 2x2x2 fine block, block voxels past the fine interior waived."""
    n = G.shape
    n2 = tuple(((m - 2 + 1) >> 1) + 2 for m in n)
    E = np.ones(tuple(2 * (m2 - 2) + 2 for m2 in n2), bool)  # fine index 0 .. 2(n2-2)+1
    c = tuple(slice(0, min(m - 1, 2 * (m2 - 2) + 2)) for m, m2 in zip(n, n2))
    E[c] = G[c]
    for ax, m in enumerate(n):  # a +1 neighbour past the fine interior (index >= m - 1) is waived
        sl = [slice(None)] * 3
        sl[ax] = slice(m - 1, None)
        E[tuple(sl)] = True
    G2 = np.zeros(n2, bool)
    core = np.ones(tuple(m2 - 2 for m2 in n2), bool)
    for a in (0, 1):
        for b in (0, 1):
            for cc in (0, 1):
                core &= E[1 + a::2, 1 + b::2, 1 + cc::2][: n2[0] - 2, : n2[1] - 2, : n2[2] - 2]
    anchor = G[1::2, 1::2, 1::2][: n2[0] - 2, : n2[1] - 2, : n2[2] - 2]
    G2[1:-1, 1:-1, 1:-1] = core & anchor
    return G2


def _band(G):
    """Boundary band B (boundary_mask_mex.c:46-132): G voxels on the outer
    interior shell or in a 2x2x2 block (odd anchors) not wholly in G, grown by
    one voxel inside G."""
    n = G.shape
    b = np.zeros(n, bool)
    inner = np.zeros(n, bool)
    inner[1:-1, 1:-1, 1:-1] = True
    shell = inner.copy()
    shell[2:-2, 2:-2, 2:-2] = False
    b |= shell & G
    full = np.ones(tuple((m - 1) // 2 for m in n), bool)  # blocks anchored at 1, 3, 5, ...
    for a in (0, 1):
        for c in (0, 1):
            for d in (0, 1):
                full &= G[1 + a::2, 1 + c::2, 1 + d::2][: full.shape[0], : full.shape[1], : full.shape[2]]
    nf = np.repeat(np.repeat(np.repeat(~full, 2, 0), 2, 1), 2, 2)
    blk = np.zeros(n, bool)
    blk[1: 1 + nf.shape[0], 1: 1 + nf.shape[1], 1: 1 + nf.shape[2]] = nf[: n[0] - 1, : n[1] - 1, : n[2] - 1]
    b |= blk & G & inner
    grown = b.copy()
    for ax in range(3):
        grown |= np.roll(b, 1, ax) | np.roll(b, -1, ax)
    return grown & G & inner


def mgpcg_fp64_ops(mask, nlevels=5, maxitmg=2, npre=2, npost=2, nb=2, coarse_outer_per_cycle=1):
    """Algorithmic floating-point operations of one PCG iteration (the
    reference's expressions, counted per updated voxel): smoothing 10 per G
    update, residual 11, restriction 30 per coarse G voxel, correction 1 add
    per fine voxel + 3.25 (mean interpolation cost) per G voxel, the
    coarsest solve's 256 sweeps per outer iteration, and the PCG vector steps
    (12 per padded voxel + 10 per G voxel for lapmg)."""
    G = np.zeros(tuple(m + 2 for m in mask.shape), bool)
    G[1:-1, 1:-1, 1:-1] = mask != 0
    levels = [G]
    for _ in range(nlevels - 1):
        levels.append(_coarsen(levels[-1]))
    vcycle = 0.0
    for l in range(nlevels - 1):
        g, bnd = float(levels[l].sum()), float(_band(levels[l]).sum())
        nint = float(np.prod([m - 2 for m in levels[l].shape]))
        bs = (1 << l) * nb
        vcycle += (npre + npost) * g * 10 + 2 * bs * bnd * 10 + 11 * g + 30 * levels[l + 1].sum() + nint + 3.25 * g
    gc = float(levels[-1].sum())
    vcycle += coarse_outer_per_cycle * (256 * gc * 10 + 11 * gc + 2 * levels[-1].size)
    n = float(G.size)
    return maxitmg * vcycle + 12 * n + 10 * float(G.sum())


def poisson_arm(qsm_gb300, ctx, torch, cpu=False):
    """256^3 MG-PCG Poisson solve with LBV's options (src/bgremove/lbv.m:58-75):
    FP64 PCG with an FP64 V-cycle (bit-identical to the oracle) beside FP64 PCG
    with an FP32 V-cycle; iterations, device time, error of the mixed solution
    against the FP64 one.  cpu: the same FP64 solve on the CPU oracle (OpenMP),
    timed, and the GPU FP64 solution compared with it bit for bit."""
    import qsm_gb300.synthetic as S

    f, mask, _ = S.config1(seed=1)
    n = f.size
    f_dev = torch.from_numpy(np.ascontiguousarray(f.transpose(2, 1, 0))).cuda()
    m_dev = torch.from_numpy(np.ascontiguousarray(mask.transpose(2, 1, 0))).cuda()
    v0 = torch.zeros_like(f_dev)
    maxit = int(np.ceil(np.sqrt(n)))
    pipe = qsm_gb300.fp_pipe_rate("float64", ctx=ctx)
    out = {"workload": "MG-PCG 256^3 FP64, rtol 1e-8, mg maxit 2, npre=npost=2, nboundary 2, mu 1, 5 levels",
           "fp64_pipe_ops_per_s": pipe}
    sols = {}
    for mixed in (False, True):
        info = {}
        qsm_gb300.mgpcg_mex(v0, f_dev, m_dev, [1, 1, 1], 1e-8, maxit, -1.0, 2, 1, 2, 2, 2, 5, mixed=mixed, ctx=ctx)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        v = qsm_gb300.mgpcg_mex(v0, f_dev, m_dev, [1, 1, 1], 1e-8, maxit, -1.0, 2, 1, 2, 2, 2, 5, mixed=mixed,
                                info=info, ctx=ctx)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        key = "fp32_vcycle" if mixed else "fp64"
        sols[key] = v
        rec = {"iters": info["iters"], "seconds": info["seconds"], "wall_s": wall, "resnorm": info["resnorm"],
               "coarse_ctas": info["coarse_ctas"], "coarse_outer": info["coarse_outer"]}
        if not mixed:
            # bound by the FP64 pipe: algorithmic FP64 operations of the solve over its time
            per_cycle = info["coarse_outer"] / max(1, 2 * info["iters"])
            ops = mgpcg_fp64_ops(mask, coarse_outer_per_cycle=per_cycle)
            rec.update(fp64_ops_per_iter=ops, fp64_ops_per_s=ops * info["iters"] / info["seconds"],
                       fp64_frac=ops * info["iters"] / info["seconds"] / pipe)
        out[key] = rec
    out["rel_l2_fp32_vcycle_vs_fp64"] = float(torch.linalg.vector_norm(sols["fp32_vcycle"] - sols["fp64"]) /
                                              torch.linalg.vector_norm(sols["fp64"]))
    out["packed_16"] = packed_poisson(qsm_gb300, ctx, torch)
    out["speedup_fp32_vcycle"] = out["fp64"]["seconds"] / out["fp32_vcycle"]["seconds"]
    if cpu:
        port = _port()
        oi = {}
        t = time.perf_counter()
        vh = port.mgpcg_mex(np.zeros_like(f, order="F"), f, mask, [1, 1, 1], 1e-8, maxit, -1.0, 2, 1, 2, 2, 2, 5,
                            info=oi)
        s = time.perf_counter() - t
        g64 = sols["fp64"].cpu().numpy().transpose(2, 1, 0)
        out["cpu_oracle"] = {"seconds": s, "iters": int(oi["iters"]), "cores": _cores(), "kind": "port",
                             "dtype": "f64", "cpu": _cpu_model(),
                             "sample": "the whole FP64 solve (FP64 V-cycle, same options), CPU oracle, OpenMP"}
        out["fp64"]["bitexact_vs_cpu_oracle"] = bool(np.array_equal(g64, vh))
        out["speedup_fp64_vs_cpu_oracle"] = s / out["fp64"]["seconds"]
        out["speedup_fp32_vcycle_vs_cpu_oracle"] = s / out["fp32_vcycle"]["seconds"]
    return out


def packed_poisson(qsm_gb300, ctx, torch, count=16, lo=96, hi=127):
    """qsm_mgpcg_batch: `count` seeded Poisson problems of lo..hi voxels per
    axis with LBV's options and the FP32 V-cycle, packed (each PCG kernel
    launched once for all), against the same solves one after another;
    results compared bit for bit."""
    import qsm_gb300.synthetic as S

    rng = np.random.default_rng(3)
    shapes = [tuple(int(x) for x in rng.integers(lo, hi + 1, 3)) for _ in range(count)]
    cases = [S.poisson_case(sh, 50 + k, semi=(lo * 0.3, lo * 0.45))[:2] for k, sh in enumerate(shapes)]
    fs = [torch.from_numpy(np.ascontiguousarray(f.transpose(2, 1, 0))).cuda() for f, _ in cases]
    ms = [torch.from_numpy(np.ascontiguousarray(m.transpose(2, 1, 0))).cuda() for _, m in cases]
    args = ([1, 1, 1], 1e-8, 200, -1.0, 2, 1, 2, 2, 2, 5)
    qsm_gb300.mgpcg_batch(None, fs, ms, *args, mixed=True, ctx=ctx)
    torch.cuda.synchronize()
    t = time.perf_counter()
    outs = qsm_gb300.mgpcg_batch(None, fs, ms, *args, mixed=True, ctx=ctx)
    torch.cuda.synchronize()
    tp = time.perf_counter() - t
    t = time.perf_counter()
    refs = [qsm_gb300.mgpcg_mex(None, f, m, *args, mixed=True, ctx=ctx) for f, m in zip(fs, ms)]
    torch.cuda.synchronize()
    ts = time.perf_counter() - t
    return {"workload": f"{count} Poisson problems {lo}..{hi} per axis (seeded), LBV options, FP32 V-cycle, 5 levels",
            "packed_s": tp, "one_by_one_s": ts, "speedup": ts / tp,
            "identical": all(bool(torch.equal(a, b)) for a, b in zip(outs, refs))}


def _generate(fn, *cols):
    """fn over the argument columns in spawned worker processes (input
    generation only; spawn is safe after CUDA initialisation)."""
    import concurrent.futures as cf
    import multiprocessing as mp

    workers = max(1, min(16, (os.cpu_count() or 1) - 1, len(cols[0])))
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(fn, *cols))


def _batch_case(b, shape):
    """Volume b of the batched configuration: the 64^3 recipe (12 ellipsoids,
    semi-axes U[4,16], chi U[-0.1,0.1] ppm, noise 0.01 ppm) at this size, in
    an inscribed ellipsoidal mask (semi-axes 0.42 x extent)."""
    import qsm_gb300.synthetic as S

    mask = S.ellipsoid_mask(shape, [0.42 * n for n in shape])
    d2f, mask, _ = S.tgv_case(shape, 3000 + b, n_ell=12, chi=(-0.1, 0.1), noise=0.01, mask=mask)
    return np.asfortranarray(d2f.astype(np.float32)), mask


def batch_arm(qsm_gb300, ctx, torch, count=32, iters=500, cpu=False):
    """Batched TV: 32 volumes of uneven size (each axis from {96..256} x
    {96..256} x {64..176} in steps of 16), lam 1e-3, 500 iterations each,
    FP32 stencils, FP64-folded monitors, all volumes in one persistent launch
    per tile shape and iteration replayed from a captured CUDA graph.  The
    tile shape per grid size comes from the autotuner (a short batch of the
    same sizes runs first and fills its table).  Against: the same volumes
    solved one after another through the one-volume fused call.  cpu: the
    CPU oracle's FP32 TV (mx_pdf of pd_tv_mex) on two of the volumes, one
    after another, timed over a 20-iteration sample each; the whole batch's
    CPU time is extrapolated from that rate."""
    import qsm_gb300.synthetic as S

    sizes = S.config3_sizes(seed=3, count=count)
    t0 = time.perf_counter()
    cases = _generate(_batch_case, list(range(count)), sizes)
    gen_s = time.perf_counter() - t0
    d2fs = [torch.from_numpy(np.ascontiguousarray(c[0].transpose(2, 1, 0))).cuda() for c in cases]
    masks = [torch.from_numpy(np.ascontiguousarray(c[1].transpose(2, 1, 0))).cuda() for c in cases]
    outs = [torch.empty_like(d) for d in d2fs]
    qsm_gb300.pd_tv_batch(d2fs, masks, [1, 1, 1], 1e-3, 0.0, 20, ctx=ctx, outs=outs)  # tunes every grid size
    infos = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    qsm_gb300.pd_tv_batch(d2fs, masks, [1, 1, 1], 1e-3, 0.0, iters, ctx=ctx, outs=outs, infos=infos)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    dev_s = infos[0]["seconds"]
    vox = sum(int(np.prod(s)) for s in sizes)
    active = sum(int(i["active_voxels"]) for i in infos)
    # algorithmic bytes are charged on the mask voxels of the interior (state moves only there)
    mask_vox = sum(int(np.count_nonzero(c[1][1:-1, 1:-1, 1:-1])) for c in cases)
    # the same volumes one after another (device time of each solve's loop)
    seq_s, same, per_vol = 0.0, True, []
    for b in range(count):
        inf = {}
        chi = qsm_gb300.pd_tv_mex(d2fs[b], masks[b], [1, 1, 1], 1e-3, 0.0, iters, fused=True, info=inf, ctx=ctx)
        seq_s += inf["seconds"]
        mv = int(np.count_nonzero(cases[b][1][1:-1, 1:-1, 1:-1]))
        per_vol.append([list(sizes[b]), mv, round(70 * mv * iters / inf["seconds"] / 1e9, 1)])
        same = same and bool(torch.equal(chi, outs[b]))
    tiles = sorted({tuple(i["tile"]) for i in infos})
    cpu_rec = None
    if cpu:
        port = _port()
        nsample, it_s = 2, 20
        t = time.perf_counter()
        for b in range(nsample):
            port.pd_tv_mex(cases[b][0], cases[b][1], [1, 1, 1], 1e-3, 0.0, it_s)
        s = time.perf_counter() - t
        rate = sum(int(np.prod(sizes[b])) for b in range(nsample)) * it_s / s
        cpu_rec = {"value": rate, "unit": "voxel-iter/s", "seconds": s, "batch_s_estimate": vox * iters / rate,
                   "cores": _cores(), "kind": "port", "dtype": "f32", "cpu": _cpu_model(),
                   "sample": f"volumes 0-{nsample - 1} ({', '.join('x'.join(map(str, sizes[b])) for b in range(nsample))}),"
                             f" {it_s} FP32 TV iterations each, one after another (CPU oracle, OpenMP)"}
    return {"cpu_oracle": cpu_rec,"workload": f"{count} TV volumes, sizes from {{96..256}}x{{96..256}}x{{64..176}} step 16, lam 1e-3, "
                        f"{iters} iterations, tol 0",
            "voxels": vox, "active_voxels": active, "iterations": iters,
            "value": vox * iters / dev_s, "unit": "voxel-iter/s",
            "device_s": dev_s, "wall_s": wall,
            "hbm_gbs": 70 * mask_vox * iters / dev_s / 1e9, "bytes_per_voxel_iter": 70, "charged_voxels": mask_vox,
            "hbm_gbs_launched_tiles": 70 * active * iters / dev_s / 1e9,
            "one_by_one_device_s": seq_s, "speedup_vs_one_by_one": seq_s / dev_s,
            "same_as_one_by_one": same, "tiles": [list(t) for t in tiles], "input_generation_s": gen_s,
            "gpu_launches_per_iteration": len(tiles),
            "one_by_one_gbs_per_volume": per_vol}


# algorithmic bytes per voxel-iteration (FP64) of the iterative next-row solvers, counting
# every array each kernel must read or write once and each FFT as one read + one write:
# TV ADMM: adj_rhs 7 arrays, D2Z 16 B, kmul 24 B, Z2D 16 B, grad_shrink 13 arrays,
# adj_norms 9 arrays; PDF/LSMR: two operator applications of 112 B (weight 3 arrays,
# R2C 16 B, spectrum multiply 24 B, C2R 16 B, Golub-Kahan update 4 arrays), two scalings
# of 2 arrays, the LSMR update 7 arrays.  FP32 anisotropic TV (the default) folds the
# two adjoint norms into the shrinkage pass (13 arrays; no 9-array norm pass):
# 7 x 4 + 8 + 12 + 8 + 13 x 4 = 108 B
TV_BYTES_F64, TV_BYTES_F32, PDF_BYTES_F64 = 288, 108, 312


def _cpu_sample(fn, iters_per_call, voxels):
    t = time.perf_counter()
    fn()
    dt = time.perf_counter() - t
    return {"value": voxels * iters_per_call / dt, "seconds": dt}


def nifti_part(qsm_gb300, ctx, torch, f4, mask, peak, cpu):
    """loadNii of a 4-echo int16 phase series (224x224x128x4, scl_slope/scl_inter,
    LPS sform: x and y flipped) into HBM as single, and saveNii of a double volume.
    The decode pass reads 2 B and writes 4 B per voxel."""
    import tempfile

    import qsm_gb300.nifti as qn

    shape = f4.shape
    n = int(np.prod(shape))
    raw = np.clip(np.round(f4 / np.abs(f4).max() * 32000), -32768, 32767).astype(np.int16)
    b = bytearray(qn.header_bytes(raw.astype(np.float32), (1, 1, 1), ctx=ctx))
    struct.pack_into("<hh", b, 70, 4, 16)                    # int16
    struct.pack_into("<ff", b, 112, float(np.abs(f4).max() / 32000), 0.0)  # scl_slope, scl_inter
    struct.pack_into("<12f", b, 280, -1, 0, 0, 224, 0, -1, 0, 224, 0, 0, 1, 0)  # LPS sform
    hdr = bytes(b)
    payload = np.asfortranarray(raw).tobytes(order="F")
    res = {"workload": "loadNii int16 224x224x128x4, scaled, LPS sform -> single in HBM; saveNii double 224x224x128"}
    dp = torch.from_numpy(np.frombuffer(payload, np.uint8).copy()).cuda()
    qn.decode(hdr, dp, device=True, ctx=ctx)
    torch.cuda.synchronize()
    reps = 20
    t = time.perf_counter()
    for _ in range(reps):
        img, _ = qn.decode(hdr, dp, device=True, ctx=ctx)
    torch.cuda.synchronize()
    sec = (time.perf_counter() - t) / reps
    res["decode_device"] = {"seconds": sec, "voxels_per_s": n / sec, "hbm_gbs": 6 * n / sec / 1e9,
                            "frac": 6 * n / sec / 1e9 / peak, "bytes_per_voxel": 6}
    with tempfile.TemporaryDirectory() as d:
        fn = os.path.join(d, "phase.nii")
        with open(fn, "wb") as fh:
            fh.write(hdr + payload)
        qn.loadNii(fn, device=True, ctx=ctx)
        t = time.perf_counter()
        for _ in range(3):
            img = qn.loadNii(fn, device=True, ctx=ctx).img
        torch.cuda.synchronize()
        sec = (time.perf_counter() - t) / 3
        res["loadNii_e2e"] = {"seconds": sec, "voxels_per_s": n / sec, "file_bytes": len(hdr) + len(payload)}
        x = torch.from_numpy(np.ascontiguousarray(f4[..., 0].T)).cuda()
        out = os.path.join(d, "chi.nii")
        t = time.perf_counter()
        for _ in range(3):
            qn.saveNii(out, x, (1, 1, 1), ctx=ctx)
        sec = (time.perf_counter() - t) / 3
        res["saveNii_e2e"] = {"seconds": sec, "voxels_per_s": x.numel() / sec}
        if cpu:
            import nifti as nio  # the oracle, for the CPU figure only

            def cpu_load():
                data = open(fn, "rb").read()
                nio.load_nii(data[:348], data[352:])
            res["cpu_oracle"] = dict(_cpu_sample(cpu_load, 1, n), unit="voxels/s", cores=1, kind="port",
                                     sample="one loadNii of the same file, numpy")
    return res


def next_rows_arm(qsm_gb300, ctx, torch, peak, cpu=True, parts="tv64,tv32,pdf,vsharp,sstgv,lbv,nifti"):
    """The widened rows on the 224x224x128 volume: TV ADMM (tv.m), PDF and V-SHARP
    background removal, the whole sstgv/lbv wrappers on 4 echoes, and NIfTI
    loading / saving.  Device solves run on resident tensors (the wrappers from
    host arrays, end to end); each CPU figure is the oracle on a bounded sample
    of the same input."""
    import qsm_gb300.synthetic as S

    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))  # the oracle, for the CPU figures
    shape = (224, 224, 128)
    n = int(np.prod(shape))
    f4, local, mask = S.field_case(shape, 7, echoes=4)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).cuda()  # noqa: E731
    m_dev = dev(mask)
    out = {"volume": list(shape), "echoes": 4}

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            r = fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t) / reps, r

    parts = set(parts.split(","))
    # TV ADMM, all iterations run (rtol = atol = 0).  FP64 is bound by the FP64 pipe
    # (cuFFT double and the FP64 stencil arithmetic), FP32 by HBM.
    it = 100
    opts = dict(maxit=it, rtol=0.0, atol=0.0)
    row = {"workload": f"tv.m ADMM, k-space data term, {it} iterations, mu 7.5e3, B0 along z"}
    for name, dt in (("f64", torch.float64), ("f32", torch.float32)):
        if "tv" + name[1:] not in parts:
            continue
        l_dev = dev(local).to(dt)
        info = {}
        sec, _ = timed(lambda: qsm_gb300.tv(l_dev, m_dev, [1, 1, 1], opts=opts, info=info, ctx=ctx))
        b = TV_BYTES_F64 if name == "f64" else TV_BYTES_F32
        row[name] = {"value": n * it / sec, "unit": "voxel-iter/s", "seconds": sec,
                     "hbm_gbs": b * n * it / sec / 1e9, "frac": b * n * it / sec / 1e9 / peak,
                     "bytes_per_voxel_iter": b}
    if cpu and "tv64" in parts:
        import tv_admm
        row["cpu_oracle"] = dict(_cpu_sample(lambda: tv_admm.tv(local, mask, [1, 1, 1], opts=dict(maxit=2, rtol=0.0,
                                                                                                    atol=0.0)), 2, n),
                                 unit="voxel-iter/s", cores=1, kind="port", sample="2 ADMM iterations, numpy FP64")
    out["tv_admm"] = row

    if cpu:
        import bgremove  # the oracle, for the CPU figures only
    if "pdf" in parts:
        # PDF: LSMR iterations on the full grid (tol 0: every iteration runs); FP64 cuFFT bound
        it = 30
        f1 = dev(f4[..., 0])
        info = {}
        sec, _ = timed(lambda: qsm_gb300.pdf(f1, m_dev, [1, 1, 1], None, [0, 0, 1], 0.0, 0.0, it, info=info,
                                             ctx=ctx))
        row = {"workload": f"pdf.m, {it} LSMR iterations, FP64", "value": n * it / sec, "unit": "voxel-iter/s",
               "seconds": sec, "hbm_gbs": PDF_BYTES_F64 * n * it / sec / 1e9,
               "frac": PDF_BYTES_F64 * n * it / sec / 1e9 / peak, "bytes_per_voxel_iter": PDF_BYTES_F64}
        if cpu:
            row["cpu_oracle"] = dict(_cpu_sample(lambda: bgremove.pdf(f4[..., 0], mask, [1, 1, 1], None, (0, 0, 1),
                                                                      0.0, 0.0, 2), 2, n),
                                     unit="voxel-iter/s", cores=1, kind="port", sample="2 LSMR iterations, numpy FP64")
        out["pdf"] = row

    if "vsharp" in parts:
        # V-SHARP, default radii (9:-2:2), 4 echoes in one call
        f4_dev = torch.from_numpy(np.ascontiguousarray(np.transpose(f4, (3, 2, 1, 0)))).cuda()
        sec, _ = timed(lambda: qsm_gb300.vsharp(f4_dev, m_dev, [1, 1, 1], ctx=ctx))
        row = {"workload": "vsharp.m, radii 9:-2:2, 4 echoes, FP64", "value": 4 * n / sec, "unit": "voxels/s",
               "seconds": sec}
        if cpu:
            row["cpu_oracle"] = dict(_cpu_sample(lambda: bgremove.vsharp(f4[..., 0], mask, [1, 1, 1]), 1, n),
                                     unit="voxels/s", cores=1, kind="port", sample="1 echo, numpy FP64")
        out["vsharp"] = row

    # whole wrappers from host arrays (crop, Laplacian, solve, scatter; echoes batched)
    if "sstgv" in parts:
        it = 300
        f4s = np.asfortranarray(f4.astype(np.float32))
        sec, _ = timed(lambda: qsm_gb300.sstgv(f4s, mask, [1, 1, 1], 1e-4, 3.0, 0.0, it, fused=True, ctx=ctx),
                       reps=2)
        out["sstgv"] = {"workload": f"sstgv.m, 4 echoes FP32 fused, {it} iterations, tol 0, host arrays",
                        "value": 4 * n * it / sec, "unit": "voxel-iter/s (dense grid)", "seconds": sec}
    if "nifti" in parts:
        out["nifti"] = nifti_part(qsm_gb300, ctx, torch, f4, mask, peak, cpu)
    if "lbv" in parts:
        infos = []
        sec, _ = timed(lambda: qsm_gb300.lbv(f4, mask, [1, 1, 1], infos=infos, ctx=ctx), reps=1)
        out["lbv"] = {"workload": "lbv.m defaults, 4 echoes FP64, host arrays", "seconds": sec,
                      "pcg_iters": [i["iters"] for i in infos], "solve_s": [i["seconds"] for i in infos],
                      "coarse_ctas": infos[0]["coarse_ctas"], "coarse_outer": [i["coarse_outer"] for i in infos]}
        # the same with the FP32 V-cycle (FP64 PCG recurrence, same stopping rule)
        mi = []
        sec_m, flm = timed(lambda: qsm_gb300.lbv(f4, mask, [1, 1, 1], mixed=True, infos=mi, ctx=ctx), reps=1)
        fl64 = qsm_gb300.lbv(f4, mask, [1, 1, 1], ctx=ctx)
        out["lbv"]["mixed"] = {"seconds": sec_m, "pcg_iters": [i["iters"] for i in mi],
                               "rel_l2_vs_fp64": float(np.linalg.norm(flm - fl64) / np.linalg.norm(fl64))}
    return out


def serve_arm(qsm_gb300, ctx, seconds=30.0, rate=4.0, per_kind=6, budget=160 * 10**9, poisson_workers=0):
    """Served reconstructions: Poisson arrivals at `rate`/s for `seconds`, 40%
    Poisson (LBV options), 30% TV (lam 1e-3, 500 iterations), 30% TGV (lam
    0.003, alpha 2, 1000 iterations), sizes as the batched configuration, a
    pool of `per_kind` seeded cases per kind, FIFO admission against a
    160 GB device budget; Poisson solves packed into the session's steps
    (poisson_workers 0) or run whole on worker threads.  Every case is first solved alone (which also tunes
    its grid size); every served result must equal its case's alone result
    bit for bit.  Errors: FP32 results against the FP64 plain GPU path (bit-
    identical to the FP64 oracle)."""
    from qsm_gb300 import serve

    t0 = time.perf_counter()
    pool = serve.make_pool(per_kind, seed=4, workers=max(1, min(16, (os.cpu_count() or 1) - 1)))
    gen_s = time.perf_counter() - t0
    alone, err = {}, {k: [] for k in serve.KINDS}
    for kind in serve.KINDS:
        for c, case in enumerate(pool[kind]):
            if kind == "poisson":
                a = serve.lbv_args(case["shape"])
                args = (None, case["f"], case["mask"], [1, 1, 1], a["tolcg"], a["maxitcg"], a["tolmg"], a["maxitmg"],
                        a["mu"], a["npre"], a["npost"], a["nboundary"], a["nlevels"])
                out = qsm_gb300.mgpcg_mex(*args, mixed=True, ctx=ctx)
                ref = qsm_gb300.mgpcg_mex(*args, mixed=False, ctx=ctx)
            elif kind == "tv":
                a = serve.TV_ARGS
                out = qsm_gb300.pd_tv_mex(case["d2f"], case["mask"], [1, 1, 1], a["lam"], a["tol"], a["maxiter"],
                                          fused=True, ctx=ctx)
                ref = qsm_gb300.pd_tv_mex(case["d2f"].astype(np.float64), case["mask"], [1, 1, 1], a["lam"], a["tol"],
                                          a["maxiter"], ctx=ctx)
            else:
                a = serve.TGV_ARGS
                out = qsm_gb300.pd_tgv_mex(case["d2f"], case["mask"], [1, 1, 1], a["lam"], a["alpha"], a["tol"],
                                           a["maxiter"], fused=True, ctx=ctx)
                ref = qsm_gb300.pd_tgv_mex(case["d2f"].astype(np.float64), case["mask"], [1, 1, 1], a["lam"],
                                           a["alpha"], a["tol"], a["maxiter"], ctx=ctx)
            alone[(kind, c)] = serve.digest(out)
            err[kind].append(float(np.linalg.norm(out.astype(np.float64) - ref) / max(np.linalg.norm(ref), 1e-300)))
    reqs = serve.arrivals(rate, seconds, seed=4, pool_size=per_kind)
    with qsm_gb300.Session(budget_bytes=budget, poisson_workers=poisson_workers, ctx=ctx) as sess:
        loop = serve.ServeLoop(sess, pool)
        recs = loop.run(reqs)
    summ = serve.summarize(recs, seconds)
    mism = [r.rid for r in recs if r.digest != alone[(r.kind, r.case)]]
    summ.update({
        "workload": f"Poisson arrivals {rate}/s for {seconds:.0f} s (seed 4), 40% Poisson / 30% TV / 30% TGV, "
                    f"sizes from {{96..256}}x{{96..256}}x{{64..176}}, {per_kind} seeded cases per kind, "
                    f"budget {budget / 1e9:.0f} GB",
        "poisson_mode": ("packed into the session steps" if poisson_workers == 0 else f"{poisson_workers} worker threads"),
        "arrived": len(reqs), "rejected": len(loop.rejected), "budget_refusals": loop.refusals,
        "max_resident": loop.max_resident, "max_queue": loop.max_queue, "steps": loop.steps,
        "same_alone_vs_mix": not mism, "mismatches": mism[:10],
        "rel_l2_vs_fp64_max": {k: (max(v) if v else None) for k, v in err.items()},
        "slowest": [{"kind": r.kind, "shape": list(r.shape), "arrive_s": round(r.t_arrive, 3),
                     "queue_ms": round(1e3 * (r.t_admit - r.t_arrive), 1),
                     "service_ms": round(1e3 * (r.t_done - r.t_admit), 1)}
                    for r in sorted(recs, key=lambda r: -r.latency)[:6]],
        "input_generation_s": gen_s})
    return summ


def _config(ws):
    return {"workload": WORKLOAD, "volume": [224, 224, 128], "iterations": ITERS, "lam": LAM, "alpha": ALPHA,
            "l2": "inputs larger than L2 (solver state ~0.93 GB per volume)", "parallelism": f"replicas x{ws}"}


def run_reference(args):
    """The reference's algorithm on the host cores: the CPU oracle (bit-exact
    with QSM.m's MEX in FP32 and FP64; the MEX files themselves need MATLAB
    and are not shipped to the GPU host) in FP32, like this benchmark's
    arm, each step a bounded iteration sample of the 1000-iteration
    inversion; one FP64 sample beside it."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    d2f, mask = _case()
    port = _port()
    d32 = np.asfortranarray(d2f.astype(np.float32))
    for _ in range(args.warmup):
        port.pd_tgv_mex(d32, mask, [1, 1, 1], LAM, ALPHA, 0.0, 2)
    budget = max(5.0, 60.0 / max(1, args.steps))
    runs = [_tgv_sample(port, d32, mask, budget) for _ in range(args.steps)]
    rates = [d2f.size * it / sec for it, sec in runs]
    v = float(np.median(rates))
    it64, s64 = _tgv_sample(port, d2f, mask, budget)
    cb = {"value": v, "unit": "voxel-iter/s", "cores": _cores(), "kind": "port", "dtype": "f32", "cpu": _cpu_model(),
          "sample": f"{runs[0][0]} of the {ITERS} FP32 iterations (mx_pdf) per step, CPU oracle, OpenMP",
          "fp64": {"value": d2f.size * it64 / s64, "unit": "voxel-iter/s",
                   "sample": f"{it64} FP64 iterations (mx_pdd), CPU oracle, OpenMP"}}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "voxel-iter/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * float(np.median([sec * ITERS / it for it, sec in runs])),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": _config(ws), "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "voxel-iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args):
    import torch

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    import qsm_gb300

    ctx = qsm_gb300.context(local)
    stream = torch.cuda.ExternalStream(qsm_gb300.lib().qsm_ctx_get_stream(ctx.handle))
    if args.only in ("batch", "serve", "next", "poisson"):
        if args.only == "batch":
            out = batch_arm(qsm_gb300, ctx, torch, cpu=not args.no_cpu and rank == 0)
        elif args.only == "poisson":
            out = poisson_arm(qsm_gb300, ctx, torch, cpu=not args.no_cpu and rank == 0)
        elif args.only == "serve":
            out = serve_arm(qsm_gb300, ctx, seconds=args.serve_seconds, rate=args.serve_rate,
                                per_kind=args.serve_pool, budget=int(args.serve_budget_gb * 1e9),
                                poisson_workers=args.serve_poisson_workers)
        else:
            out = next_rows_arm(qsm_gb300, ctx, torch, _peaks()[0], cpu=not args.no_cpu, parts=args.next_parts)
        if rank == 0:
            print(json.dumps({"profile_run": True, args.only: out}))
        return
    ITERS = args.iters
    d2f, mask = _case(tuple(int(v) for v in args.shape.split(",")) if args.shape else None)
    N = d2f.size
    shape_c = d2f.shape[::-1]
    # device-resident inputs (C-order (nz, ny, nx) tensors == MATLAB x-fastest)
    d2f_dev = torch.from_numpy(np.ascontiguousarray(d2f.transpose(2, 1, 0))).cuda()
    mask_dev = torch.from_numpy(np.ascontiguousarray(mask.transpose(2, 1, 0))).cuda()

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    def timed(fn, steps):
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = None
        for _ in range(steps):
            out = fn()
        e1.record(stream)
        barrier()
        return max_over_ranks(e0.elapsed_time(e1), dist, "cuda"), out

    info = {}

    def mixed_step():
        return qsm_gb300.pd_tgv_mex(d2f_dev, mask_dev, [1, 1, 1], LAM, ALPHA, 0.0, ITERS, fused=True, info=info, ctx=ctx)

    for _ in range(args.warmup):
        mixed_step()
    with ClockSampler(local) as clk:
        ms, chi_mixed = timed(mixed_step, args.steps)
    loop_s = info["seconds"]
    value = whole_job_rate(N * ITERS * args.steps, ws, ms * 1e-3)
    if args.only == "fused":
        if rank == 0:
            print(json.dumps({"profile_run": True, "value": value, "unit": "voxel-iter/s", "shape": list(d2f.shape),
                              "iters": ITERS, "loop_s": loop_s, "tile": list(info["tile"]),
                              "active_voxels": int(info["active_voxels"])}))
        return

    # fused-kernel roofline: average launch time from the library's loop events; the
    # algorithmic bytes are charged on the mask voxels of the interior (the voxels whose state
    # the kernel reads and writes: outside the mask it moves none)
    peak, peak_kind = _peaks()
    t_launch = loop_s / info["iters"]
    active = int(info["active_voxels"])  # voxels of the launched (mask-holding) tiles
    mask_vox = int(np.count_nonzero(mask[1:-1, 1:-1, 1:-1]))
    achieved = ALG_BYTES_FP32 * mask_vox / t_launch / 1e9
    digest = kernel_digest()
    traffic = None if args.shape else NCU_TRAFFIC_224x224x128.get((digest,) + tuple(info["tile"]))

    # plain FP64 path (reference structure, bit-exact with the reference MEX)
    d2f64_dev = d2f_dev
    info64 = {}

    def plain_step():
        return qsm_gb300.pd_tgv_mex(d2f64_dev, mask_dev, [1, 1, 1], LAM, ALPHA, 0.0, ITERS, info=info64, ctx=ctx)

    plain_step()
    ms64, chi64 = timed(plain_step, max(1, min(2, args.steps)))
    value64 = whole_job_rate(N * ITERS * max(1, min(2, args.steps)), ws, ms64 * 1e-3)
    rel = float(torch.linalg.vector_norm(chi_mixed - chi64) / torch.linalg.vector_norm(chi64))

    # end to end through the C ABI with pinned host buffers
    h_d2f = torch.empty(shape_c, dtype=torch.float64, pin_memory=True)
    h_d2f.copy_(d2f_dev.cpu())
    h_mask = torch.empty(shape_c, dtype=torch.uint8, pin_memory=True)
    h_mask.copy_(mask_dev.cpu())
    h_chi = torch.empty(shape_c, dtype=torch.float64, pin_memory=True)
    # (nx, ny, nz) Fortran-ordered numpy views of the pinned buffers
    np_d2f, np_mask, np_chi = h_d2f.numpy().T, h_mask.numpy().T, h_chi.numpy().T

    def e2e_step():
        return qsm_gb300.pd_tgv_mex(np_d2f, np_mask, [1, 1, 1], LAM, ALPHA, 0.0, ITERS, fused=True, ctx=ctx, out=np_chi)

    e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
    e2e_value = whole_job_rate(N * ITERS * args.steps, ws, e2e_s)

    cpu_rank0 = not args.no_cpu and rank == 0
    poisson = None if args.no_poisson else poisson_arm(qsm_gb300, ctx, torch, cpu=cpu_rank0)
    batch = None if args.no_batch else batch_arm(qsm_gb300, ctx, torch, cpu=cpu_rank0)
    served = None if args.no_serve else serve_arm(qsm_gb300, ctx, seconds=args.serve_seconds, rate=args.serve_rate,
                                per_kind=args.serve_pool, budget=int(args.serve_budget_gb * 1e9),
                                poisson_workers=args.serve_poisson_workers)
    nxt = None if args.no_next else next_rows_arm(qsm_gb300, ctx, torch, peak, cpu=not args.no_cpu and rank == 0)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    cb, rel_oracle = None, None
    if not args.no_cpu:
        cb, chi_oracle = cpu_baseline(d2f, mask)
        cm = chi_mixed.cpu().numpy().transpose(2, 1, 0)
        rel_oracle = float(np.linalg.norm(cm - chi_oracle) / np.linalg.norm(chi_oracle))
    line = {
        "metric": METRIC, "value": value, "unit": "voxel-iter/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (FP64-folded monitors)", "data": "synthetic",
        "config": _config(ws),
        "fp64_plain": {"value": value64, "unit": "voxel-iter/s", "ms_per_step": ms64 / max(1, min(2, args.steps))},
        "speedup_vs_fp64": value / value64, "rel_l2_vs_fp64": rel,
        # the FP64 oracle's own chi (CPU, all 1000 iterations); the plain FP64 GPU path is bit-identical to it
        "rel_l2_vs_fp64_oracle": rel_oracle,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "bytes_per_voxel_iter": ALG_BYTES_FP32, "charged_voxels": mask_vox,
                     "charged_voxels_rule": "mask voxels of the interior (state read and written there only)",
                     "traffic": traffic / 1e9 if traffic else None,
                     "traffic_unit": "GB per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum)",
                     "frac_dram": traffic / t_launch / 1e9 / peak if traffic else None,
                     "traffic_note": None if traffic else
                     f"no ncu capture recorded for this kernel build (digest {digest}) and tile",
                     "kernel_digest": digest,
                     "kernel": ("stream_k<%d,%d,TGV> z-chunk %d" if info["tile"][0] == 28 else "tgv_fused_k<%d,%d,%d>")
                               % tuple(info["tile"]),
                     "avg_launch_us": t_launch * 1e6, "peak_source": peak_kind,
                     "achieved_launched_tiles": ALG_BYTES_FP32 * active / t_launch / 1e9,
                     "launched_tile_voxels": active, "tile": list(info["tile"]), "dense_voxels": N},
        "cpu_baseline": cb,
        "e2e": {"value": e2e_value, "unit": "voxel-iter/s", "h2d_bytes_per_step": int(N * 8 + N),
                "d2h_bytes_per_step": int(N * 8)},
        "poisson": poisson,
        "batch": batch,
        "served": served,
        "next_rows": nxt,
        "gpu_launches": int(args.steps * (ITERS + 5)),
        "clocks": clk.summary(),
    }
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    # profiling aids (the reported configuration uses the defaults)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-poisson", action="store_true", help="skip the MG-PCG arm")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched TV arm")
    ap.add_argument("--no-serve", action="store_true", help="skip the served-requests arm")
    ap.add_argument("--no-next", action="store_true", help="skip the TV ADMM / background removal / wrapper arm")
    ap.add_argument("--next-parts", default="tv64,tv32,pdf,vsharp,sstgv,lbv,nifti",
                    help="parts of the next-rows arm with --only next (profiling aid)")
    ap.add_argument("--serve-seconds", type=float, default=30.0, help="arrival window of the served arm")
    ap.add_argument("--serve-rate", type=float, default=4.0, help="arrivals per second of the served arm")
    ap.add_argument("--serve-pool", type=int, default=6, help="seeded input cases per request kind (served arm)")
    ap.add_argument("--serve-budget-gb", type=float, default=160.0, help="device byte budget of the served arm")
    ap.add_argument("--serve-poisson-workers", type=int, default=0,
                    help="served arm: 0 packs Poisson solves into the session steps, N > 0 runs them on N threads")
    ap.add_argument("--shape", default="", help="nx,ny,nz of a reduced volume (profiler captures)")
    ap.add_argument("--iters", type=int, default=ITERS, help="iterations per inversion (profiler captures)")
    ap.add_argument("--only", default="all", choices=["all", "fused", "batch", "serve", "next", "poisson"],
                    help="run only one arm (profiling aid)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
