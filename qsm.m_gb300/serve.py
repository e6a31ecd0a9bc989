"""Request loop for served QSM reconstructions on one GPU.

Requests (Poisson/LBV solves, TV and TGV inversions of uneven volume sizes)
arrive as a Poisson process.  The loop keeps a FIFO of arrived requests and
admits the head whenever a slot is free and its device footprint fits in
the session's byte budget (the session refuses a submit that does not fit
with QSM_ERR_BUSY and the request waits).  Admitted solves stay resident on
the device: primal-dual solves advance together in 30-iteration batched
steps; Poisson solves advance in the same steps (packed launches, a session
without Poisson workers) or run on worker streams at the same time; and a
request that arrives while others are running joins the next step
(continuous batching).  Finished results are fetched as soon as they are done; latency
is arrival to fetched result.

The session is any object with the :class:`qsm_gb300.Session` methods, and
the clock and sleep are injectable, so the admission and accounting logic
runs unchanged against a fake session on a CPU.

The reference has no serving layer (QSM.m processes one volume per MATLAB
call); the solves behind each request are pd_tv_mex / pd_tgv_mex
(src/inversion/sstgv.m:83-87) and mgpcg_mex with the LBV options
(src/bgremove/lbv.m:58-75, :108-113).
"""
from __future__ import annotations

import collections
import dataclasses
import hashlib
import math
import time

import numpy as np

KINDS = ("poisson", "tv", "tgv")

# solver arguments per kind
TV_ARGS = dict(lam=1e-3, tol=0.0, maxiter=500)
TGV_ARGS = dict(lam=0.003, alpha=2.0, tol=0.0, maxiter=1000)


def lbv_args(shape):
    """mgpcg options of lbv.m:58-75: tol 1e-8, maxit ceil(sqrt(N)), mg maxit 2,
    npre = npost = 2, nboundary 2, mu 1, 5 levels."""
    n = int(np.prod(shape))
    return dict(tolcg=1e-8, maxitcg=int(math.ceil(math.sqrt(n))), tolmg=-1.0, maxitmg=2, mu=1, npre=2, npost=2,
                nboundary=2, nlevels=5)


@dataclasses.dataclass
class Request:
    rid: int
    t_arrive: float      # seconds after the start of the loop
    kind: str            # "poisson" | "tv" | "tgv"
    case: int            # index into the input pool of its kind


@dataclasses.dataclass
class Record:
    rid: int
    kind: str
    case: int
    shape: tuple
    t_arrive: float
    t_admit: float
    t_done: float
    digest: str          # sha256 of the result bytes
    iters: int
    device_s: float = 0.0  # the solve's device time as the session reports it (see summarize)

    @property
    def latency(self) -> float:
        return self.t_done - self.t_arrive


def arrivals(rate: float, duration: float, seed: int, mix=(0.4, 0.3, 0.3), pool_size: int = 8) -> list[Request]:
    """A Poisson arrival stream (exponential gaps of mean 1/rate) over
    [0, duration); each request draws its kind from `mix` (poisson, tv, tgv)
    and one of `pool_size` seeded input cases of that kind."""
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            return out
        kind = KINDS[int(rng.choice(3, p=np.asarray(mix) / np.sum(mix)))]
        out.append(Request(len(out), float(t), kind, int(rng.integers(pool_size))))


def pool_case(kind: str, shape, case_seed: int) -> dict:
    """One seeded input case (see make_pool)."""
    from . import synthetic

    shape = tuple(int(n) for n in shape)
    if kind == "poisson":
        f, m, _ = synthetic.poisson_case(shape, case_seed, semi=(0.3 * min(shape), 0.45 * min(shape)))
        return dict(shape=shape, f=f, mask=m)
    mask = synthetic.ellipsoid_mask(shape, [0.42 * n for n in shape])
    d2f, mask, _ = synthetic.tgv_case(shape, case_seed, n_ell=12, chi=(-0.1, 0.1), noise=0.01, mask=mask)
    return dict(shape=shape, d2f=d2f.astype(np.float32, order="F"), mask=mask)


def make_pool(per_kind: int, seed: int, sizes=None, workers: int = 1) -> dict:
    """Seeded inputs: per kind `per_kind` cases with volume sizes drawn as in
    the batched configuration (each axis from {96..256}x{96..256}x{64..176}
    in steps of 16).  PD cases: an ellipsoid phantom and its field as in the
    64^3 configuration (noise 0.01 ppm) in an inscribed ellipsoidal mask;
    Poisson cases: the 256^3 Poisson recipe at that size.  workers > 1
    generates in spawned processes (safe after CUDA initialisation)."""
    from . import synthetic

    jobs = []
    for ki, kind in enumerate(KINDS):
        shp = sizes or synthetic.config3_sizes(seed=seed + 10 * ki, count=per_kind)
        for c in range(per_kind):
            jobs.append((kind, tuple(shp[c % len(shp)]), seed * 1000 + ki * 100 + c))
    if workers > 1:
        import concurrent.futures as cf
        import multiprocessing as mp

        with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
            cases = list(ex.map(pool_case, *zip(*jobs)))
    else:
        cases = [pool_case(*j) for j in jobs]
    pool = {k: [] for k in KINDS}
    for (kind, _, _), case in zip(jobs, cases):
        pool[kind].append(case)
    return pool


def footprint(kind: str, shape) -> int:
    from . import footprint as fp

    return fp({"poisson": "mgpcg", "tv": "tv", "tgv": "tgv"}[kind], shape, 5)


def submit(session, req: Request, case: dict) -> int:
    """Submits one request; raises QsmError(BUSY) if it does not fit."""
    if req.kind == "poisson":
        a = lbv_args(case["shape"])
        return session.submit_mgpcg(None, case["f"], case["mask"], [1, 1, 1], a["tolcg"], a["maxitcg"], a["tolmg"],
                                    a["maxitmg"], a["mu"], a["npre"], a["npost"], a["nboundary"], a["nlevels"],
                                    mixed=True)
    if req.kind == "tv":
        a = TV_ARGS
        return session.submit_pd(case["d2f"], case["mask"], [1, 1, 1], a["lam"], 0.0, a["tol"], a["maxiter"],
                                 tgv=False)
    a = TGV_ARGS
    return session.submit_pd(case["d2f"], case["mask"], [1, 1, 1], a["lam"], a["alpha"], a["tol"], a["maxiter"],
                             tgv=True)


def digest(a) -> str:
    a = np.asarray(a)
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def is_busy(err: Exception) -> bool:
    return getattr(err, "status", None) == 8  # QSM_ERR_BUSY


class ServeLoop:
    """FIFO admission by slots and device footprint, continuous batched
    stepping, retirement as soon as a result is done."""

    def __init__(self, session, pool: dict, *, max_active: int = 64, step_iters: int = 30,
                 clock=time.perf_counter, sleep=time.sleep, keep_results: bool = False):
        self.s = session
        self.pool = pool
        self.max_active = max_active
        self.step_iters = step_iters
        self.clock = clock
        self.sleep = sleep
        self.keep_results = keep_results
        self.results: dict[int, np.ndarray] = {}
        self.records: list[Record] = []
        self.refusals = 0         # submits refused for lack of budget
        self.rejected: list[Request] = []  # larger than the whole budget
        self.max_resident = 0     # most requests resident at once
        self.max_queue = 0        # longest FIFO of waiting requests
        self.steps = 0

    def run(self, reqs: list[Request]) -> list[Record]:
        pending = collections.deque(sorted(reqs, key=lambda r: r.t_arrive))
        queue: collections.deque[Request] = collections.deque()
        active: dict[int, tuple[Request, float]] = {}
        t0 = self.clock()
        while pending or queue or active:
            now = self.clock() - t0
            while pending and pending[0].t_arrive <= now:
                queue.append(pending.popleft())
            self.max_queue = max(self.max_queue, len(queue))
            # admission: FIFO, while a slot is free and the head fits
            while queue and len(active) < self.max_active:
                r = queue[0]
                try:
                    jid = submit(self.s, r, self.pool[r.kind][r.case])
                except Exception as e:  # noqa: BLE001
                    if not is_busy(e):
                        raise
                    self.refusals += 1
                    if not active:
                        # refused with nothing resident: it can never fit
                        self.rejected.append(queue.popleft())
                        continue
                    break
                queue.popleft()
                active[jid] = (r, self.clock() - t0)
            self.max_resident = max(self.max_resident, len(active))
            # a session without Poisson workers advances its resident Poisson solves in its steps
            steps_poisson = getattr(self.s, "poisson_workers", 1) == 0
            pd_running = any(r.kind != "poisson" or steps_poisson for r, _ in active.values())
            if pd_running:
                self.s.step(self.step_iters)
                self.steps += 1
            # retire everything that is done
            for jid in list(active):
                fin, info = self.s.poll(jid)
                if not fin:
                    continue
                r, t_admit = active.pop(jid)
                out = self.s.fetch(jid)
                t_done = self.clock() - t0
                case = self.pool[r.kind][r.case]
                self.records.append(Record(r.rid, r.kind, r.case, tuple(case["shape"]), r.t_arrive, t_admit, t_done,
                                           digest(out), int(info.get("iters", 0)), float(info.get("seconds", 0.0))))
                if self.keep_results and (r.kind, r.case) not in self.results:
                    self.results[(r.kind, r.case)] = out
            if not pd_running:
                # nothing to step: wait for the next arrival or a Poisson worker
                nxt = pending[0].t_arrive - (self.clock() - t0) if pending else 0.0
                if active:
                    self.sleep(0.0005)
                elif not queue and nxt > 0:
                    self.sleep(min(nxt, 0.05))
        return self.records


def summarize(records: list[Record], duration: float) -> dict:
    """p50/p99 latency (ms) overall and per kind, throughput (requests/s)."""
    if not records:
        return dict(requests=0)
    lat = np.array([r.latency for r in records]) * 1e3
    span = max(max(r.t_done for r in records), duration)
    out = dict(requests=len(records), p50_ms=float(np.percentile(lat, 50)), p99_ms=float(np.percentile(lat, 99)),
               mean_ms=float(lat.mean()), throughput_rps=len(records) / span, span_s=span)
    for k in KINDS:
        lk = np.array([r.latency for r in records if r.kind == k]) * 1e3
        if lk.size:
            # device_s: Poisson jobs, the solve's span on its worker stream; primal-dual jobs, the
            # batched steps they took part in (shared with the other jobs of those steps)
            dev = float(sum(r.device_s for r in records if r.kind == k))
            out[k] = dict(n=int(lk.size), p50_ms=float(np.percentile(lk, 50)), p99_ms=float(np.percentile(lk, 99)),
                          device_s=dev, device_share_of_span=dev / span)
    return out
