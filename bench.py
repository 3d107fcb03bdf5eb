"""Benchmark of the GB300 Henon step: star-updates/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--N stars]

Workload (N = 1 GPU): King W0 = 6 cluster, N = 1e6 stars, Kroupa (2001) IMF
masses, single stars, FP64 plain step (sort -> potential -> relaxation -> new
orbits, with the time step, Stodolkiewicz energy conservation and tidal
stripping between them), seeded synthetic input.  One "step" is one whole
Henon step of every star; one star-update is one star carried through it.
The state (about 250 bytes/star, 250 MB) is larger than the 129 MB L2, so
every step streams from HBM; no explicit L2 flush is needed.

The same line carries the N = 1e7 configuration (King W0 = 7, 10% composite
binaries, FP32 relaxation kinematics) and the 128-cluster ensemble as
sub-objects, each with its own throughput, roofline, energy drift and the
learned proposal's numbers.

--impl reference times the reference's algorithm on the host cores instead:
the oracle's C restatement (bit-identical to the reference's own step compiled
against single-rank shims; the full reference needs MPI, GSL and HDF5, which
this image lacks), with the reference's own taus113 generator, one process per
core, each stepping the same model the GPU arm steps.

Under torchrun each rank steps its own replica (replicas only: the path has
no data exchange between independent clusters) and value is the sum over
ranks of star-updates divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "cmc-cosmic_gb300"))

METRIC = "star-updates/s per Henon step"
UNIT = "star-updates/s"
# algorithmic HBM bytes per star for each kernel family (compulsory FP64 SoA
# traffic: reads + writes of the fields the phase consumes and produces)
ALG_BYTES = {"sort": 116, "potential": 24, "relax": 72, "orbit": 80, "ec3": 72, "energy": 56,
             "timestep": 24, "tidal": 16, "begin": 0, "end": 0, "mlp": 0}
# the proposal network's algorithmic FLOPs per star: 2 (8*64 + 64*64 + 64*33)
MLP_FLOPS_PER_STAR = 2 * (8 * 64 + 64 * 64 + 64 * 33)
# DRAM bytes per star of one launch, dram__bytes_read.sum + dram__bytes_write.sum
# from one-kernel, one-launch ncu captures on the King W0=6 + Kroupa model at
# N = 1e6 (962,913 stars in the captured step): k_orbit 142.4 MB, k_relax64
# 58.0 MB, k_ec3 63.1 MB, k_sort_gather 97.6 MB
NCU_TRAFFIC_PER_STAR = {"orbit": 142.4e6 / 962913, "relax": 58.0e6 / 962913, "ec3": 63.1e6 / 962913}
# share of cycles the FP64 pipe was busy in the same captures: the kernels'
# real bound on GB300, reported beside the HBM roofline
NCU_FP64_PIPE_ACTIVE = {"orbit": 0.742, "relax": 0.838, "ec3": 0.845, "potential": 0.816, "timestep": 0.705}
# FP64 thread-operations per star of each kernel family
# (smsp__sass_thread_inst_executed_op_fp64_pred_on.sum over the stars of one
# step, same model: k_orbit 338.2 and k_orbit_pre 8.0, k_relax64 168.3, k_ec3
# 45.0, k_timestep 12.1), and the FP64 pipe's rate at 100% busy, ops / (time x
# busy) from those captures: 4.7-5.6e11 thread-operations/s
NCU_FP64_OPS_PER_STAR = {"orbit": 346.2, "relax": 168.3, "potential": 61.4, "ec3": 45.0, "energy": 11.8,
                         "timestep": 12.1, "tidal": 2.1}
FP64_PEAK_OPS = 5.05e11


def measured_peak(key="hbm_gbs", fallback=6800.0):
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d[key]), "measured"
    except Exception:
        return fallback, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0, None
    import torch
    import torch.distributed as dist

    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", "0"))
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend=backend)
    return rank, ws, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allreduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# The named synthetic configurations (seeded generators; no dataset exists for
# them).  king1e6 is the headline; king1e7bin and ensemble128 are measured
# beside it in the same line (EXTRA_CONFIGS); the others on request.
CONFIGS = {
    "plummer1e5": dict(model="plummer", N=100_000, imf=0, bf=0.0, fp32=0,
                       desc="Plummer, equal masses, N=1e5, plain FP64 Henon step"),
    "king1e6": dict(model="king", w0=6.0, N=1_000_000, imf=1, bf=0.0, fp32=0,
                    desc="King W0=6, Kroupa IMF, N=1e6, plain FP64 Henon step"),
    "ensemble128": dict(model="ensemble", n=128, lo=10_000, hi=1_000_000, imf=1, bf=0.0, fp32=0,
                        desc="128 clusters, N log-uniform in [1e4,1e6], alternating Plummer / King W0 in "
                             "{3,5,7,9}, Kroupa IMF, one launch per kernel, whole step in a CUDA graph, FP64"),
    "king4e6": dict(model="king", w0=7.0, N=4_000_000, imf=1, bf=0.0, fp32=0,
                    desc="King W0=7, Kroupa IMF, N=4e6, plain FP64 Henon step (plain sampler)"),
    "king1e7bin": dict(model="king", w0=7.0, N=10_000_000, imf=1, bf=0.1, fp32=1,
                       desc="King W0=7, Kroupa IMF, N=1e7, 10% composite binaries, FP32 relaxation "
                            "kinematics with FP64 energies, FP64 potential and root finds"),
}


EXTRA_CONFIGS = ("king1e7bin", "ensemble128")
MODEL_SEED = 20240607  # the model every arm builds (plus the rank under torchrun)


def make_model(N: int, seed: int, cfg=None):
    import cmcgpu

    cfg = cfg or CONFIGS["king1e6"]
    if cfg["model"] == "plummer":
        return cmcgpu.generate(cmcgpu.PLUMMER, N, seed=seed, imf=cfg["imf"], binary_fraction=cfg["bf"])
    return cmcgpu.generate(cmcgpu.KING, N, seed=seed, w0=cfg.get("w0", 6.0), imf=cfg["imf"],
                           binary_fraction=cfg["bf"])


def make_clusters(cfg, N, rank):
    """[(N_c, ic, seed)] for the configuration: one cluster, or the ensemble
    (per-cluster seeds derived from one master seed)."""
    import numpy as np

    import cmcgpu

    if cfg["model"] != "ensemble":
        return [(N, make_model(N, MODEL_SEED + rank, cfg), cmcgpu.derive_seed(777, rank))]
    from concurrent.futures import ThreadPoolExecutor

    master = MODEL_SEED + rank
    rng = np.random.default_rng(master)
    Ns = np.exp(rng.uniform(np.log(cfg["lo"]), np.log(cfg["hi"]), cfg["n"])).astype(int)
    w0s = rng.choice([3.0, 5.0, 7.0, 9.0], cfg["n"])

    def one(i):
        seed = cmcgpu.derive_seed(master, i)
        if i % 2 == 0:
            ic = cmcgpu.generate(cmcgpu.PLUMMER, int(Ns[i]), seed=seed, imf=cfg["imf"])
        else:
            ic = cmcgpu.generate(cmcgpu.KING, int(Ns[i]), seed=seed, w0=float(w0s[i]), imf=cfg["imf"])
        return int(Ns[i]), ic, seed

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        return list(ex.map(one, range(cfg["n"])))


def workload_config(cfg_name: str, N: int):
    """The `config` object both arms print: what is stepped, nothing about how."""
    cfg = CONFIGS[cfg_name]
    n = N or cfg.get("N")
    state = (n or 28_000_000) * 250
    return {"workload": cfg["desc"], "name": cfg_name, "N": n if cfg["model"] != "ensemble" else None,
            "model_seed": MODEL_SEED,
            "l2": "state ~250 B/star exceeds the 129 MB L2: no flush needed" if state > 129e6
                  else "L2 holds the state: steps read warm data"}


# ------------------------------------------------------------- CPU legs ---
def _ref_worker(args):
    """One host core: the oracle (reference algorithm, taus113 draws) stepping
    the workload's model (the ensemble: its largest King member's kind);
    returns (stars*steps, seconds)."""
    n, steps, warmup, draw_seed, cfg_name = args
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "cmc-cosmic_gb300"))
    import oracle

    cfg = CONFIGS[cfg_name]
    if cfg["model"] == "ensemble":
        cfg = dict(CONFIGS["king1e6"], w0=5.0)
    ic = make_model(n, MODEL_SEED, cfg)
    o = oracle.Oracle(ic, oracle.default_params(orbit_r=ic["rtid"], seed=draw_seed,
                                                draw_mode=oracle.DRAW_TAUS113))
    o.initialize()
    for _ in range(warmup):
        o.step()
    t0 = time.perf_counter()
    done = 0
    for _ in range(steps):
        done += o.nstars()
        o.step()
    return done, time.perf_counter() - t0


def cpu_baseline(n_sample: int, steps: int, warmup: int, procs: int, cfg_name: str = "king1e6"):
    """The oracle on `procs` host processes (spawned: no GPU state is forked),
    each stepping the workload's model; star-updates/s over the slowest."""
    import multiprocessing as mp

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.build()
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        res = pool.map(_ref_worker, [(n_sample, steps, warmup, 1000 + i, cfg_name) for i in range(procs)])
    updates = sum(r[0] for r in res)
    secs = max(r[1] for r in res)
    return updates / secs, secs


# ------------------------------------------------------ learned proposal ---
def train_proposal(a):
    """The orbit sampler's proposal network, trained as the learned
    configuration specifies: records (features, accepted X, trials) of the
    plain sampler on the Plummer N=1e5 model, Adam at lr 1e-3, batch 8192."""
    import numpy as np

    import cmcgpu

    cfg = CONFIGS["plummer1e5"]
    N = cfg["N"]
    ic = make_model(N, 20240611, cfg)
    g = cmcgpu.Context([N], cmcgpu.default_params(orbit_r=ic["rtid"], seed=cmcgpu.derive_seed(779, 0)))
    g.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    g.initialize()
    g.set_learned(cmcgpu.LEARN_COLLECT)
    t0 = time.perf_counter()
    feats, bins, nts = [], [], []
    n = 0
    while n < a.learn_records:
        g.step(1)
        f, X, nt = g.learned_samples()
        feats.append(f)
        bins.append(np.minimum((X * 32).astype(np.int32), 31))
        nts.append(nt)
        n += len(X)
    g.check_device("collect")
    feat, b, nt = np.concatenate(feats), np.concatenate(bins), np.concatenate(nts)
    t1 = time.perf_counter()
    g.mlp_init(7)
    loss = g.mlp_train(feat, b, nt, steps=a.learn_steps, batch=8192, lr=1e-3, seed=11)
    w = g.mlp_params()
    t2 = time.perf_counter()
    g.close()
    return w, {"records": int(len(b)), "model": "Plummer N=1e5 (plain sampler)", "adam_steps": a.learn_steps,
               "batch": 8192, "lr": 1e-3, "plain_trials_per_star": float(nt.mean()),
               "loss_first": [float(x) for x in loss[:20].mean(axis=0)],
               "loss_last": [float(x) for x in loss[-100:].mean(axis=0)],
               "collect_s": round(t1 - t0, 2), "train_s": round(t2 - t1, 2),
               # forward + backward (3x the forward's FLOPs) per record, whole training call
               "train_tflops": 3 * MLP_FLOPS_PER_STAR * 8192 * a.learn_steps / max(t2 - t1, 1e-9) / 1e12}


def learned_leg(a, clusters, params, ctx, timed, stars, w):
    """Learned-proposal step on the same context (after the plain legs), the
    cost of a trial from a sweep of envelope factors, and one step from a
    common state with each sampler for the distribution test."""
    import numpy as np
    from scipy.stats import ks_2samp

    import cmcgpu

    ctx.mlp_set_params(w)
    ctx.set_learned(cmcgpu.LEARN_ON, a.kappa)
    tuned = ctx.autotune(2) if not a.no_autotune else "off"
    ctx.use_graph(True)
    ctx.step(a.warmup)
    ctx.check_device("learned warmup")
    n0 = stars()
    ncl = len(clusters)
    e_start = [ctx.scalar("Etot", c) for c in range(ncl)]
    ms, launches = timed(a.steps, True)
    ctx.check_device("learned steps")
    drift = [(ctx.scalar("Etot", c) - e0) / abs(e0) / a.steps for c, e0 in enumerate(e_start)]
    st = ctx.learned_stats()
    ctx.profile(True)
    ctx.kernel_time("reset")
    timed(a.steps, False)
    fam = {name: ctx.kernel_time(name) for name in ALG_BYTES}
    # what any proposal could save: the orbit phase's time against trials per
    # star, over envelope factors (the proposal's trials and nothing else
    # change), fitted by a line; its slope is the marginal cost of a trial
    sweep = []
    for kappa in (1.05, a.kappa, 1.6, 2.4):
        ctx.set_learned(cmcgpu.LEARN_ON, kappa)
        ctx.step(1)
        ctx.kernel_time("reset")
        timed(a.steps, False)
        ms_orb = ctx.kernel_time("orbit")[0] / a.steps
        s_k = ctx.learned_stats()
        tps = (s_k["trials"] + s_k["plain_trials"]) / max(s_k["accepted"] + s_k["plain_stars"], 1)
        sweep.append((kappa, tps, ms_orb))
    ctx.profile(False)
    ctx.set_learned(cmcgpu.LEARN_OFF)
    slope, icept = np.polyfit([t for _, t, _ in sweep], [m for _, _, m in sweep], 1)
    mlp_ms = fam["mlp"][0] / max(fam["mlp"][1], 1)
    # the network runs inside a long step: the sustained BF16 rate is its peak
    peak, peak_kind = measured_peak("bf16_tflops_sustained", 1700.0)
    achieved = MLP_FLOPS_PER_STAR * n0 / (mlp_ms * 1e-3) / 1e12
    # the same state through both samplers: one step each
    n, ic, seed = clusters[0]
    pair = []
    for mode in (cmcgpu.LEARN_COLLECT, cmcgpu.LEARN_ON):
        g = cmcgpu.Context([n], [params[0]])
        g.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
        g.initialize()
        g.mlp_set_params(w)
        g.set_learned(mode, a.kappa)
        g.step(1)
        g.check_device("learned pair")
        _, X, nt = g.learned_samples()
        pair.append((X, nt, g.learned_stats()))
        g.close()
    (Xa, nta, _), (Xb, _, stb) = pair
    trials = (stb["trials"] + stb["plain_trials"]) / max(stb["accepted"] + stb["plain_stars"], 1)
    return {
        "what": "orbit sampler with the learned proposal (exact rejection against min(g, F) under "
                "kappa F P q; envelope failures go back to the plain sampler)",
        "kappa": a.kappa,
        "value": n0 * a.steps / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / a.steps,
        "gpu_launches": launches,
        "energy": {"rel_drift_per_step": drift[0] if ncl == 1 else None,
                   "max_abs_rel_drift_per_step": max(abs(d) for d in drift)},
        "autotune": tuned,
        "trials_per_star": trials, "plain_trials_per_star": float(nta.mean()),
        "failed_frac": stb["failed"] / max(stb["stars"], 1),
        "ks_p_X": float(ks_2samp(Xa, Xb).pvalue), "ks_samples": [int(len(Xa)), int(len(Xb))],
        "ks_cluster": "cluster 0" if ncl > 1 else "the cluster",
        "last_step_stats": st,
        "kernels": {k: {"ms_per_step": round(v[0] / a.steps, 4), "launches": v[1]} for k, v in fam.items() if v[1]},
        "mlp_roofline": {"bound": "tensor", "kernel": "k_mlp_infer", "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved / peak, "peak_source": peak_kind + " (bf16 sustained)",
                         "flops_per_star": MLP_FLOPS_PER_STAR, "ms_per_launch": mlp_ms},
        "trial_cost": {
            "what": "orbit-phase ms per step against trials per star over envelope factors kappa (a line fit): "
                    "the slope is the marginal cost of one more trial per star; a proposal that needed one trial "
                    "per star and cost nothing could save at most slope * (plain trials - 1) of the plain step",
            "sweep": [{"kappa": k, "trials_per_star": t, "orbit_ms": m} for k, t, m in sweep],
            "ms_per_trial_per_star": float(slope), "orbit_ms_at_zero_trials": float(icept),
            "max_saving_ms": float(slope * (float(nta.mean()) - 1.0)),
        },
    }


def fp32_error_leg(cluster, params):
    """FP32 relaxation kinematics against FP64: one relaxation from the same
    state with each, per-output errors (velocities against the star's speed)."""
    import numpy as np

    import cmcgpu

    n, ic, seed = cluster
    out = {}
    for fp32 in (0, 1):
        p = cmcgpu.default_params(orbit_r=ic["rtid"], seed=seed, relax_fp32=fp32)
        g = cmcgpu.Context([n], [p])
        g.load(0, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
        g.initialize()
        g.begin_step()
        g.calc_timestep()
        g.dynamics_apply(g.scalar("Dt"))
        g.check_device("fp32 leg")
        out[fp32] = {k: g.get(k) for k in ("vr_rel", "vt_rel", "E", "J")}
        out[fp32]["r"] = g.get("star_r")[1:len(out[fp32]["E"]) + 1]
        g.close()
    a, b = out[0], out[1]
    speed = np.sqrt(a["vr_rel"] ** 2 + a["vt_rel"] ** 2)
    return {"what": "one relaxation from the same state, FP32 kinematics against FP64, max over stars: "
                    "velocities against the star's speed, E relative, J against r times the speed",
            "vr_over_speed": float(np.max(np.abs(b["vr_rel"] - a["vr_rel"]) / speed)),
            "vt_over_speed": float(np.max(np.abs(b["vt_rel"] - a["vt_rel"]) / speed)),
            "E_rel": float(np.max(np.abs(b["E"] - a["E"]) / np.abs(a["E"]))),
            "J_over_r_speed": float(np.max(np.abs(b["J"] - a["J"]) / (a["r"] * speed)))}


def trig32_leg(a, clusters, tuned_relax):
    """The same clusters with cmcg_params.relax_trig32 (the relaxation's sines
    and cosines on the FP32 pipe): the graph-replayed step timed with CUDA
    events over the same number of steps, and the relaxation's own time from a
    profiled run of them."""
    import torch

    import cmcgpu

    params = [cmcgpu.default_params(orbit_r=ic["rtid"], seed=seed, relax_trig32=1) for _, ic, seed in clusters]
    g = cmcgpu.Context([n for n, _, _ in clusters], params)
    for c, (n, ic, _) in enumerate(clusters):
        g.load(c, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    g.initialize()
    g.use_graph(True)
    g.step(a.warmup)
    g.check_device("trig32 warm-up")
    stream = torch.cuda.ExternalStream(g.stream_handle())
    n0 = sum(g.nstars(c) for c in range(len(clusters)))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g.synchronize()
    e0.record(stream)
    g.step(a.steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    g.check_device("trig32 steps")
    g.use_graph(False)
    g.profile(True)
    g.kernel_time("reset")
    g.step(a.steps)
    g.synchronize()
    relax_ms = g.kernel_time("relax")[0] / a.steps
    g.close()
    return {"what": "relax_trig32 = 1: the FP64 relaxation's sines and cosines in double-float on the FP32 pipe "
                    "(within 2e-14 of sin/cos; off by default)",
            "value": n0 * a.steps / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / a.steps,
            "relax_ms_per_step": relax_ms, "default_relax_ms_per_step": tuned_relax}


# ------------------------------------------------------------ GPU leg ----
def measure(a, cfg_name, N, rank, ws, dist, weights=None, sub=False):
    """One configuration on this rank's GPU: the device-resident step replayed
    from the CUDA graph (value), the kernel families and the roofline of the
    top one, the public host-array API end to end (e2e), the energy drift, and
    with `weights` the learned proposal's step."""
    import torch

    import cmcgpu

    cfg = CONFIGS[cfg_name]
    N = N or cfg.get("N", 0)
    clusters = make_clusters(cfg, N, rank)
    params = [cmcgpu.default_params(orbit_r=ic["rtid"], seed=seed, relax_fp32=cfg["fp32"]) for _, ic, seed in clusters]
    ctx = cmcgpu.Context([n for n, _, _ in clusters], params)
    for c, (n, ic, _) in enumerate(clusters):
        ctx.load(c, ic["r"], ic["m"], ic["vr"], ic["vt"], ic["id"])
    ctx.initialize()
    ncl = len(clusters)

    def stars():
        return sum(ctx.nstars(c) for c in range(ncl))

    stream = torch.cuda.ExternalStream(ctx.stream_handle())

    def timed(k, graph):
        """k steps between CUDA events recorded on the context's stream."""
        ctx.use_graph(graph)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier(dist)
        ctx.synchronize()
        e0.record(stream)
        ctx.step(k)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), ctx.launch_count()

    # launch variants picked by measurement on this context (real steps)
    tuned = ctx.autotune(2) if not a.no_autotune else "off"
    # warm-up in the timed mode (the first step captures the graph)
    ctx.use_graph(True)
    ctx.step(a.warmup)
    ctx.check_device("warmup")
    n_start = stars()

    # ---- device-resident steps replayed from the CUDA graph
    e_start = [ctx.scalar("Etot", c) for c in range(ncl)]
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    time.sleep(0.6)
    ms, launches = timed(a.steps, True)
    clk = clocks.stop()
    ctx.check_device("timed steps")
    # total energy (compute_energy_new's Etot, escaped energy included) per step
    drift = [(ctx.scalar("Etot", c) - e0) / abs(e0) / a.steps for c, e0 in enumerate(e_start)]
    ms_max = allreduce_max(dist, ms)
    updates = allreduce_sum(dist, float(n_start * a.steps))
    value = updates / (ms_max * 1e-3)

    # ---- the same number of steps launched directly, with CUDA events per kernel family
    n_prof = stars()
    ctx.profile(True)
    ctx.kernel_time("reset")
    ms_prof, _ = timed(a.steps, False)
    ctx.check_device("profiled steps")
    fam = {name: ctx.kernel_time(name) for name in ALG_BYTES}
    ctx.profile(False)
    step_ms = sum(v[0] for v in fam.values()) / a.steps
    top = max((k for k in fam if ALG_BYTES[k] > 0), key=lambda k: fam[k][0])
    ms_top, n_top = fam[top]
    peak, peak_kind = measured_peak()
    achieved = ALG_BYTES[top] * n_prof / (ms_top / n_top * 1e-3) / 1e9
    per_family = {k: {"ms_per_step": round(v[0] / a.steps, 4), "launches": v[1]} for k, v in fam.items() if v[1]}
    step_bytes = sum(ALG_BYTES.values()) - ALG_BYTES["ec3"] - ALG_BYTES["energy"] - ALG_BYTES["timestep"] \
        - ALG_BYTES["tidal"]  # the four hot-path kernels' 292 B per star-update

    # ---- end to end through the public API: host star arrays in pinned
    # memory, copied in before and out after every step (cmcg_step_host)
    def pinned(n):
        b = {k: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for k in ("r", "m", "vr", "vt", "E", "J")}
        b["id"] = torch.empty(n, dtype=torch.int64, pin_memory=True).numpy()
        return b

    bufs, ns = [], []
    for c, (n, _, _) in enumerate(clusters):
        b = pinned(n + 16)
        bufs.append(b)
        ns.append(ctx.get_stars(c, b))
    hs = cmcgpu.HostStars(bufs, ns)  # steps in place on the same arrays
    ctx.use_graph(True)
    ns = ctx.step_host_inplace(hs)  # captures the part graphs
    h2d = d2h = 0
    e2e_updates = 0
    barrier(dist)
    t1 = time.perf_counter()
    for _ in range(a.steps):
        h2d += sum(ns) * 7 * 8
        d2h += sum(ns) * 7 * 8 + 8 * ncl
        e2e_updates += sum(ns)
        ns = ctx.step_host_inplace(hs)
    e2e_dt = time.perf_counter() - t1
    barrier(dist)
    ctx.check_device("e2e steps")
    e2e_value = allreduce_sum(dist, float(e2e_updates)) / allreduce_max(dist, e2e_dt)

    out = {
        "value": value,
        "unit": UNIT,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": ms_max / a.steps,
        "stars_at_start": n_start,
        "clusters": ncl,
        "autotune": tuned,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d // a.steps,
                "d2h_bytes_per_step": d2h // a.steps},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": (NCU_TRAFFIC_PER_STAR[top] * n_prof if top in NCU_TRAFFIC_PER_STAR else None),
                     "fp64_pipe_active": NCU_FP64_PIPE_ACTIVE.get(top),
                     "alg_bytes_per_star": ALG_BYTES[top], "ms_per_launch": ms_top / n_top,
                     "step_frac": step_bytes * value / ws / 1e9 / peak,
                     "timed_in": "the profiled direct-launch pass"},
        "roofline_fp64": {"bound": "fp64 pipe", "kernel": top,
                          "achieved": NCU_FP64_OPS_PER_STAR.get(top, 0.0) * n_prof / (ms_top / n_top * 1e-3),
                          "peak": FP64_PEAK_OPS, "unit": "FP64 ops/s",
                          "frac": NCU_FP64_OPS_PER_STAR.get(top, 0.0) * n_prof / (ms_top / n_top * 1e-3)
                          / FP64_PEAK_OPS,
                          "ops_per_star": NCU_FP64_OPS_PER_STAR.get(top),
                          "peak_source": "the FP64 pipe at 100% busy, from the ncu captures (4.7-5.6e11 ops/s)",
                          "step_frac": sum(NCU_FP64_OPS_PER_STAR.values()) * n_prof / (step_ms * 1e-3)
                          / FP64_PEAK_OPS},
        "energy": {"rel_drift_per_step": drift[0] if ncl == 1 else None,
                   "max_abs_rel_drift_per_step": max(abs(d) for d in drift),
                   "what": "(Etot after - Etot before) / |Etot before| / steps over the timed steps"},
        "kernels": per_family,
        "kernel_ms_per_step": step_ms,
        "profiled_ms_per_step": ms_prof / a.steps,
        "clocks": clk,
    }
    if weights is not None and rank == 0 and ws == 1:
        try:
            out["learned"] = learned_leg(a, clusters, params, ctx, timed, stars, weights)
            out["learned"]["speedup_vs_plain"] = out["learned"]["value"] / value
            tc = out["learned"]["trial_cost"]
            plain_ms = ms_max / a.steps
            # Amdahl: the plain step less the most any proposal could save
            tc["max_speedup_any_proposal"] = plain_ms / max(plain_ms - tc["max_saving_ms"], 1e-9)
        except Exception as e:  # the plain numbers stand without it
            out["learned"] = {"error": repr(e)}
    ctx.close()
    if cfg["fp32"] and rank == 0:
        out["fp32_vs_fp64"] = fp32_error_leg(clusters[0], params)
    if not cfg["fp32"] and not sub and rank == 0 and ws == 1:
        try:
            out["relax_trig32"] = trig32_leg(a, clusters, per_family.get("relax", {}).get("ms_per_step"))
            out["relax_trig32"]["speedup_vs_default"] = out["relax_trig32"]["value"] / value
        except Exception as e:  # the default numbers stand without it
            out["relax_trig32"] = {"error": repr(e)}
    return out


def run_ours(a, rank, ws, dist):
    import cmcgpu

    cmcgpu.build()
    weights, train_info = None, None
    if not a.no_learned and rank == 0 and ws == 1:
        try:
            weights, train_info = train_proposal(a)
        except Exception as e:
            train_info = {"error": repr(e)}
    m = measure(a, a.config, a.N, rank, ws, dist, weights)
    cfg = CONFIGS[a.config]
    model_txt = {"plummer": "Plummer model", "king": f"King W0={cfg.get('w0')} model",
                 "ensemble": "Plummer and King models"}[cfg["model"]]
    out = {
        "metric": METRIC,
        "value": m["value"],
        "unit": UNIT,
        "n_gpus": ws,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": m["ms_per_step"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if not cfg["fp32"] else "f64 (f32 relaxation kinematics)",
        "data": f"synthetic (seeded {model_txt}, {'Kroupa 2001 IMF' if cfg['imf'] else 'equal masses'}; no dataset)",
        "config": workload_config(a.config, a.N),
        "run": {"clusters": m["clusters"], "stars_at_start": m["stars_at_start"], "parallelism": f"replicas x{ws}",
                "timing": "CUDA events on the library's stream; whole step replayed from a CUDA graph"},
        "autotune": m["autotune"],
        "e2e": m["e2e"],
        "gpu_launches": m["gpu_launches"],
    }
    for k in ("roofline", "roofline_fp64", "energy", "kernels", "kernel_ms_per_step", "profiled_ms_per_step",
              "clocks", "learned", "fp32_vs_fp64", "relax_trig32"):
        if k in m:
            out[k] = m[k]
    if train_info is not None:
        out.setdefault("learned", {})["train"] = train_info
    if not a.no_extra and a.config == "king1e6" and not a.N and ws == 1:
        out["configs"] = {}
        for name in EXTRA_CONFIGS:
            try:
                sub = measure(a, name, 0, rank, ws, dist, weights)
                sub["config"] = workload_config(name, 0)
                out["configs"][name] = sub
            except Exception as e:  # the headline stands without them
                out["configs"][name] = {"error": repr(e)}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="king1e6", choices=sorted(CONFIGS))
    ap.add_argument("--N", type=int, default=0, help="override the configuration's N (single-cluster configs)")
    ap.add_argument("--cpu-sample", type=int, default=1_000_000, help="stars per CPU-baseline process")
    ap.add_argument("--cpu-steps", type=int, default=3, help="timed oracle steps of the 1-core CPU baseline")
    ap.add_argument("--cpu-warmup", type=int, default=1, help="untimed oracle steps before them")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip training the proposal network and timing the learned-proposal step")
    ap.add_argument("--no-extra", action="store_true",
                    help="measure the headline configuration alone (not king1e7bin and ensemble128 beside it)")
    ap.add_argument("--kappa", type=float, default=1.2, help="envelope factor of the learned proposal")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch variants")
    ap.add_argument("--learn-records", type=int, default=20_000_000, help="plain-sampler records to train on")
    ap.add_argument("--learn-steps", type=int, default=2500, help="Adam steps of batch 8192")
    a = ap.parse_args()
    if a.warmup < 3:
        a.warmup = 3
    rank, ws, local, dist = dist_setup()

    if a.impl == "reference":
        if rank != 0:  # the CPU arm runs on rank 0 alone; the other ranks leave without work
            if dist is not None:
                dist.destroy_process_group()
            return
        procs = min(os.cpu_count() or 1, 16)
        cfg = CONFIGS[a.config]
        n_sample = a.cpu_sample if cfg["model"] == "ensemble" else (a.N or cfg.get("N"))
        n_sample = min(n_sample, a.cpu_sample)
        val, secs = cpu_baseline(n_sample, a.steps, a.warmup, procs, a.config)
        out = {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
               "ms_per_step": secs / a.steps * 1e3, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "impl": "reference",
               "data": "synthetic (seeded cluster models of the configuration; no dataset)",
               "config": workload_config(a.config, a.N),
               "cpu_baseline": {"value": val, "unit": UNIT, "cores": procs, "kind": "port",
                                "sample": f"{procs} processes, each stepping a {n_sample}-star cluster of the "
                                          f"configuration's model (model seed {MODEL_SEED}), {a.warmup} warm-up + "
                                          f"{a.steps} timed steps (the oracle, bit-identical to the reference's "
                                          f"compiled step; taus113 draws)"},
               "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        if dist is not None:
            dist.destroy_process_group()
        return

    out = run_ours(a, rank, ws, dist)
    if rank == 0:
        if not a.no_cpu_baseline and ws == 1:
            cfg = CONFIGS[a.config]
            n_sample = min(a.cpu_sample, a.N or cfg.get("N") or a.cpu_sample)
            val, secs = cpu_baseline(n_sample, a.cpu_steps, a.cpu_warmup, 1, a.config)
            out["cpu_baseline"] = {"value": val, "unit": UNIT, "cores": 1, "kind": "port",
                                   "sample": f"one {n_sample}-star cluster of the configuration's model (model seed "
                                             f"{MODEL_SEED}), {a.cpu_warmup} warm-up + {a.cpu_steps} timed steps "
                                             f"({secs:.1f} s; the oracle, bit-identical to the reference's compiled "
                                             f"step, taus113 draws, 1 core)"}
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
