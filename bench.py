"""Benchmark: ensemble member-steps/s for forward + adjoint at M=42, B=256.

One bench "step" is one complete differentiable integration of the workload:
B = 256 forced members at M = 42 (64 x 128 grid), 1440 modified-Euler time
steps forward, then the hand-written adjoint steps back to gradients of the loss
mean((Phi_T - Phi_target)^2) with respect to the initial (eta, delta, Phi,
U, V) and to taurad, taudrag, DPhieq and Phibar of every member.  The adjoint
gets its primal states as the library's Integration decides (--store auto):
the FP32 run keeps all 1441 states (154 GB of HBM) and needs no
recomputation; the FP64 run (twice the bytes) checkpoints every 50 steps and
recomputes each window.  --store checkpoint forces the recomputing form.
The ensemble runs as two groups of 128 members of one plan, each group's step
chain on its own stream (--groups, swp_plan_set_concurrency): the groups'
latency-bound kernels overlap; the results equal those of joint launches.

value : fast path (FP32 state and pointwise math) on device-resident inputs,
        B * 1440 / seconds per step.  The plain FP64 GPU path is timed on the
        same workload and reported beside it with the error of the fast path
        against it (relative L2 and max of eta, delta, Phi after 1440 steps).
e2e   : the same metric through the public API (torch.autograd over
        my_swampe_gb300.adjoint.integrate) with pinned HOST inputs copied in
        and the gradients copied out inside the timed region.
--impl reference : the reference's CPU algorithm (the oracle restatement, run
        with torch autograd on the host cores) on a bounded sample of the
        same workload.

The data are synthetic (my_swampe_gb300.workloads.forced_ensemble).  One
integration touches far more than L2 (154 GB of stored states, or ~9 GB of
checkpoints and window slots); L2 is also flushed with a 512 MB write between
timed steps.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

METRIC = "ensemble steps/s fwd+adjoint at M=42, fast vs plain FP64 GPU, at stated error"
UNIT = "member-steps/s"
M_BENCH, B_BENCH, T_BENCH, CKPT = 42, 256, 1440, 50


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def _tensor_peak():
    """Dense bf16 TFLOP/s (burst), measured or the fallback."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["bf16_tflops"]), "measured"
        except Exception:
            pass
    return 1900.0, "fallback"


# Algorithmic Legendre FLOPs of one member-step at M=42 (forward; the adjoint
# transposes the same transforms): 18 distinct complex transforms (11 forward,
# 7 inverse), each 4 J sum_m (M + 1 - m) = 4 * 64 * 946 real flops.
LEGENDRE_FLOP_M42 = 18 * 4 * 64 * 946


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200",
                                          "-i", str(_local_rank())], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "", 1).isdigit())
        mx = max(float(r[2]) for r in rows if r[2].replace(".", "", 1).isdigit())
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(rows)}


def _local_rank():
    return int(os.environ.get("LOCAL_RANK", "0"))


def _flush_l2(buf):
    buf.add_(1.0)


def _group_sizes(B, ngroups):
    sizes = [B // ngroups] * ngroups
    sizes[-1] += B - sum(sizes)
    return sizes


def _setup(precision, B, seed=1234, store="auto", ngroups=2, M=M_BENCH, autotune=True):
    """The B-member ensemble as `ngroups` groups of one plan, run concurrently
    (one stream per group); member b keeps its seed (seed + b) whatever the split."""
    from my_swampe_gb300.engine import Engine, RunFlagsC
    from my_swampe_gb300.adjoint import Integration
    from my_swampe_gb300 import workloads

    sizes = _group_sizes(B, ngroups)
    # the project's autotuner picks each group's Legendre kernel (tensor cores or a SIMT tile)
    eng = Engine([(M, b) for b in sizes], precision, concurrent=ngroups > 1, autotune=autotune)
    wls, off = [], 0
    for g, b in enumerate(sizes):
        wl = workloads.forced_ensemble(eng, g=g, seed=seed + off)
        workloads.apply_params(eng, g, wl["params"])
        wls.append(wl)
        off += b
    flags = RunFlagsC()
    integ = Integration(eng, flags, t0=2, nsteps=T_BENCH, ckpt_every=CKPT, store=store)
    ics = [wl["ics"].to(eng.rdtype) for wl in wls]
    return eng, wls, flags, integ, ics


def _target(eng, wls, flags, ics):
    """Phi_target per group: a run at perturbed taurad (x1.1) and DPhieq (x0.9)."""
    from my_swampe_gb300 import workloads

    for g, wl in enumerate(wls):
        p = dict(wl["params"])
        p["taurad"] = p["taurad"] * 1.1
        p["DPhieq"] = p["DPhieq"] * 0.9
        workloads.apply_params(eng, g, p)
    eng.init_state(ics, flags)
    eng.forward(flags, t0=2, nsteps=T_BENCH)
    tgt = [o[2].clone() for o in eng.output_physical(flags)]
    for g, wl in enumerate(wls):
        workloads.apply_params(eng, g, wl["params"])
    return tgt


def _one_step(integ, ics, targets):
    """forward + adjoint of the loss mean over all members of (Phi_T - target)^2;
    device-resident.  Returns per-group lists."""
    import torch

    outs = integ.run_forward(ics)
    n = sum(t.numel() for t in targets)
    ds = []
    for out, tgt in zip(outs, targets):
        d = torch.zeros_like(out)
        d[2] = (2.0 / n) * (out[2] - tgt)
        ds.append(d)
    dic, grad = integ.run_backward(ds)
    return outs, dic, grad


def shard_seed(rank: int, base: int = 1234) -> int:
    """Seed of rank `rank`'s member shard: every rank integrates its own B
    members (member b of rank r is drawn from shard_seed(r) + b)."""
    return base + 100000 * int(rank)


def reduce_max_time(t: float, world: int, device) -> float:
    """The job's time: the maximum over ranks of the per-rank time (the only
    collective of the N > 1 bench; the data path has none)."""
    if world <= 1:
        return float(t)
    import torch
    import torch.distributed as dist

    tt = torch.tensor([float(t)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def job_throughput(world: int, B: int, steps: int, t_max: float) -> float:
    """Whole-job member-steps/s: all ranks' members over the slowest rank's time."""
    return world * B * steps / t_max


def _time_steps(fn, steps, warmup, flush):
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        flush()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    return times


def _algorithmic_bytes(kernel, B, J=64, M=42, elem=8):
    """Algorithmic DRAM bytes of one launch: Fourier columns (J x (M+1) complex
    per member) each kernel must read and write.
      spectral : reads 11 step inputs + 3 RA-filtered carries, writes 3 curr + U, V + 3 carries
      grid     : reads eta, Phi, U, V; writes A..E, PhiF, F, G
      grid_adj : reads 4 primal + 6 lambda(A..E, PhiF; those of F, G equal B, -A) + 3 lambda(eta,
                 delta, Phi outputs; those of U, V are zero inside a sweep); writes 5
      spectral_adj : reads 5 lambda(outputs) + 7 primal inputs; writes 11 lambda fields (the
                 other 8 stay zero inside a sweep)"""
    cols = {"spectral": 22, "grid": 12, "grid_adj": 18, "spectral_adj": 23}[kernel]
    return cols * J * (M + 1) * elem * B


# ncu summary (profiles/) of each kernel at this workload, which records the
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch
_PROFILE_OF = {"spectral": "k_spectral_tc_fast_M42_B256.md", "grid": "k_grid_step_fast_M42_B256.md",
               "grid_adj": "k_grid_adjoint_fast_M42_B256.md", "spectral_adj": "k_spectral_adj_tc_fast_M42_B256.md"}


def _ncu_traffic(kernel):
    """DRAM bytes per launch of `kernel` from its committed ncu summary (the line
    'traffic_bytes_per_launch: N'), or None when there is no capture."""
    p = ROOT / "profiles" / _PROFILE_OF.get(kernel, "")
    if not p.is_file():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return int(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def run_ours(args):
    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(_local_rank())
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from __graft_entry__ import build

    # one rank per node compiles (if anything is stale); the others wait for it
    if _local_rank() == 0:
        build()
    if world > 1:
        torch.distributed.barrier()
    if _local_rank() != 0:
        build()  # loads the library (nothing left to compile)
    B = args.B
    peak, peak_kind = _peaks()
    flush_buf = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    flush = lambda: _flush_l2(flush_buf)  # noqa: E731

    # ---------------- fast path (headline)
    ng = args.groups
    eng, wls, flags, integ, ics = _setup("fast", B, seed=shard_seed(rank), store=args.store, ngroups=ng)
    target = _target(eng, wls, flags, ics)
    state = {}

    def step_fast():
        state["out"], state["dic"], state["grad"] = _one_step(integ, ics, target)

    if world > 1:
        torch.distributed.barrier()
    sampler = ClockSampler()
    sampler.start()
    times = _time_steps(step_fast, args.steps, args.warmup, flush)
    clocks = sampler.stop()
    t_max = reduce_max_time(float(np.mean(times)), world, "cuda")
    value = job_throughput(world, B, T_BENCH, t_max)
    out_fast = torch.cat([o.double() for o in state["out"]], dim=1)
    grad_fast = torch.cat([g.clone() for g in state["grad"]], dim=1)

    # kernel roofline (CUDA events inside the library on the launching stream)
    kt = eng.time_kernels(flags, nrep=20, adjoint=True)
    per_step = {k: v for k, v in kt.items()}
    # per model step of fwd+adjoint: the adjoint kernels run once; the forward ones
    # once with stored states, twice (forward + window recompute) with checkpoints
    nfwd = 1 if integ.store == "all" else 2
    share = {"spectral": nfwd * per_step["spectral"], "grid": nfwd * per_step["grid"],
             "grid_adj": per_step["grid_adj"], "spectral_adj": per_step["spectral_adj"]}
    dom = max(share, key=share.get)
    alg = _algorithmic_bytes(dom, B, elem=8)
    achieved = alg / (per_step[dom] * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_kind": peak_kind, "traffic": _ncu_traffic(dom),
                "ms_per_launch": {k: round(v, 5) for k, v in per_step.items()},
                "algorithmic_bytes_per_launch": alg}
    # every kernel against HBM; the Legendre kernels also in algorithmic TFLOP/s
    # against the dense bf16 peak (their 3xTF32 MMAs issue about 2.5x these flops)
    tpeak, tpeak_kind = _tensor_peak()
    per_kernel = {}
    for k, ms in per_step.items():
        ab = _algorithmic_bytes(k, B, elem=8)
        gbs = ab / (ms * 1e-3) / 1e9
        e = {"ms": round(ms, 5), "algorithmic_bytes": ab, "gbs": round(gbs, 1), "frac_hbm": round(gbs / peak, 4)}
        if k in ("spectral", "spectral_adj"):
            fl = LEGENDRE_FLOP_M42 * B
            tf = fl / (ms * 1e-3) / 1e12
            e.update(algorithmic_flop=fl, tflops=round(tf, 2), frac_tensor_bf16=round(tf / tpeak, 5))
        per_kernel[k] = e
    roofline["per_kernel"] = per_kernel
    roofline["tensor_peak_tflops"] = tpeak
    roofline["tensor_peak_kind"] = tpeak_kind

    # ---------------- e2e through the public API with host buffers
    from my_swampe_gb300.adjoint import integrate, GRAD_PARAMS, Integration

    sizes = _group_sizes(B, ng)
    host_ics = [x.detach().cpu().pin_memory() for x in ics]
    host_par = []
    for g, wl in enumerate(wls):
        hp = {k: wl["params"][k].detach().cpu().pin_memory() for k in GRAD_PARAMS if k != "Phibar"}
        hp["Phibar"] = torch.full((sizes[g],), wl["params"]["Phibar"], dtype=torch.float64).pin_memory()
        host_par.append(hp)
    host_tgt = [t.detach().cpu().pin_memory() for t in target]
    out_ic = [torch.empty(x.shape, dtype=x.dtype).pin_memory() for x in host_ics]
    out_par = [torch.empty((4, b), dtype=torch.float64).pin_memory() for b in sizes]
    n_tgt = sum(t.numel() for t in host_tgt)

    def step_e2e():
        d_ics = [x.to("cuda", non_blocking=True).requires_grad_(True) for x in host_ics]
        d_par = [{k: v.to("cuda", non_blocking=True).requires_grad_(True) for k, v in hp.items()} for hp in host_par]
        d_tgt = [t.to("cuda", non_blocking=True) for t in host_tgt]
        outs = integrate(eng, flags, 2, T_BENCH, d_par, d_ics, ckpt_every=CKPT, integration=integ)
        loss = sum(((o[2].double() - t.double()) ** 2).sum() for o, t in zip(outs, d_tgt)) / n_tgt
        loss.backward()
        for g in range(ng):
            out_ic[g].copy_(d_ics[g].grad, non_blocking=True)
            for k, name in enumerate(GRAD_PARAMS):
                out_par[g][k].copy_(d_par[g][name].grad, non_blocking=True)

    e2e_times = _time_steps(step_e2e, max(2, args.steps), 1, flush)
    e2e_t = reduce_max_time(float(np.mean(e2e_times)), world, "cuda")
    h2d = sum(x.numel() * x.element_size() for x in host_ics) + \
        sum(v.numel() * 8 for hp in host_par for v in hp.values()) + \
        sum(t.numel() * t.element_size() for t in host_tgt)
    d2h = sum(x.numel() * x.element_size() for x in out_ic) + sum(x.numel() * 8 for x in out_par)

    store_fast = integ.store
    integ.release()
    del integ, step_e2e, step_fast
    torch.cuda.empty_cache()

    # ---------------- e2e through the drop-in API: run_model_scan_final with tensors
    # that require grad, torch.autograd backward, host buffers in and out
    dropin_e2e = None
    if not args.skip_dropin:
        from my_swampe_gb300 import run_model_scan_final

        d_host_ics = [torch.cat([x[k] for x in host_ics], 0).pin_memory() for k in range(5)]  # (B, J, I) each
        d_host_par = {k: torch.cat([hp[k] for hp in host_par], 0).pin_memory() for k in GRAD_PARAMS}
        d_host_tgt = torch.cat([t for t in host_tgt], 0).pin_memory()
        d_out_ic = [torch.empty(x.shape, dtype=x.dtype).pin_memory() for x in d_host_ics]
        d_out_par = torch.empty((4, B), dtype=torch.float64).pin_memory()
        wl0 = wls[0]["params"]

        def step_dropin():
            xs = [x.to("cuda", non_blocking=True).requires_grad_(True) for x in d_host_ics]
            pr = {k: v.to("cuda", non_blocking=True).requires_grad_(True) for k, v in d_host_par.items()}
            tg = d_host_tgt.to("cuda", non_blocking=True)
            r = run_model_scan_final(M=M_BENCH, dt=float(wl0["dt"]), tmax=2 + T_BENCH, Phibar=pr["Phibar"],
                                     omega=float(wl0["omega"]), a=float(wl0["a"]), taurad=pr["taurad"],
                                     taudrag=pr["taudrag"], DPhieq=pr["DPhieq"], K6=float(wl0["K6"]),
                                     eta0_init=xs[0], delta0_init=xs[1], Phi0_init=xs[2], U0_init=xs[3],
                                     V0_init=xs[4], precision="fast")
            loss = ((r["last_state"].Phi_curr.double() - tg.double()) ** 2).sum() / tg.numel()
            loss.backward()
            for k in range(5):
                d_out_ic[k].copy_(xs[k].grad, non_blocking=True)
            for k, name in enumerate(GRAD_PARAMS):
                d_out_par[k].copy_(pr[name].grad, non_blocking=True)

        di_times = _time_steps(step_dropin, max(2, args.steps), 1, flush)
        di_t = reduce_max_time(float(np.mean(di_times)), world, "cuda")
        di_h2d = sum(x.numel() * x.element_size() for x in d_host_ics) + sum(v.numel() * 8 for v in
                                                                             d_host_par.values()) + \
            d_host_tgt.numel() * d_host_tgt.element_size()
        di_d2h = sum(x.numel() * x.element_size() for x in d_out_ic) + d_out_par.numel() * 8
        dropin_e2e = {"value": round(job_throughput(world, B, T_BENCH, di_t), 1), "unit": UNIT,
                      "h2d_bytes_per_step": int(di_h2d), "d2h_bytes_per_step": int(di_d2h),
                      "ms_per_step": round(1e3 * di_t, 3),
                      "api": "my_swampe_gb300.run_model_scan_final (differentiable) + torch.autograd backward, "
                             "B members (run as two concurrent halves)"}
        del step_dropin
        torch.cuda.empty_cache()
    # ---------------- fast path with the FP64 run's state policy (checkpoints + recompute),
    # so the FP64 speed-up can also be read at equal algorithm
    fast_ckpt = None
    if not args.skip_fp64 and store_fast != "checkpoint":
        integ_c = Integration(eng, flags, t0=2, nsteps=T_BENCH, ckpt_every=CKPT, store="checkpoint")
        tc_ = _time_steps(lambda: _one_step(integ_c, ics, target), 2, 1, flush)
        fast_ckpt = world * B * T_BENCH / float(np.mean(tc_))
        integ_c.release()
        del integ_c
        torch.cuda.empty_cache()
    # ---------------- plain FP64 GPU path on the same workload
    fp64 = None
    if not args.skip_fp64:
        eng64, wl64, flags64, integ64, ics64 = _setup("fp64", B, seed=shard_seed(rank), store=args.store,
                                                      ngroups=ng)
        target64 = [t.double() for t in target]
        st64 = {}

        def step64():
            st64["out"], st64["dic"], st64["grad"] = _one_step(integ64, ics64, target64)

        t64 = _time_steps(step64, args.fp64_steps, 1, flush)
        v64 = B * T_BENCH / float(np.mean(t64))
        o64 = torch.cat(st64["out"], dim=1)
        err = {}
        for k, name in enumerate(("eta", "delta", "Phi")):
            ref = o64[k]
            dif = out_fast[k] - ref
            err[name] = {"rel_l2": float(torch.linalg.vector_norm(dif) / torch.linalg.vector_norm(ref)),
                         "max_abs": float(dif.abs().max()), "max_rel_to_fieldmax": float(dif.abs().max() / ref.abs().max())}
        g64 = torch.cat(st64["grad"], dim=1)
        gerr = {name: float(torch.linalg.vector_norm(grad_fast[k] - g64[k]) / torch.linalg.vector_norm(g64[k]))
                for k, name in enumerate(GRAD_PARAMS)}
        kt64 = eng64.time_kernels(flags64, nrep=5, adjoint=True)
        fp64 = {"value": round(v64, 1), "ms_per_step": round(1e3 * float(np.mean(t64)), 3), "steps": args.fp64_steps,
                "adjoint_states": integ64.store,
                "speedup_fast_over_fp64": round(value / (world * v64), 2),
                "fast_with_checkpoint_states": None if fast_ckpt is None else round(fast_ckpt, 1),
                "speedup_at_equal_state_policy": round((fast_ckpt if fast_ckpt else value) / (world * v64), 2),
                "error_fast_vs_fp64_after_1440": err,
                "grad_rel_l2_fast_vs_fp64": gerr,
                "ms_per_launch": {k: round(v, 5) for k, v in kt64.items()},
                # the FP64 Legendre kernel against the chip's FP64 (non-tensor) rate:
                # SMs x 2 DFMA x 2 FLOP x the SM clock under load
                "legendre_fp64_tflops": round(LEGENDRE_FLOP_M42 * B / (kt64["spectral"] * 1e-3) / 1e12, 3),
                "fp64_peak_tflops_nominal": round(_fp64_peak_tflops(clocks), 3)}

    # ---------------- other workloads: the drop-in API's forward rate, the mixed-truncation ensemble
    dropin = None if args.skip_dropin else _dropin_leg()
    mixed = None if args.skip_mixed else _mixed_leg()
    emission = None if args.skip_emission else _emission_leg()

    # ---------------- CPU baseline (oracle restatement, torch autograd, host cores)
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        cpu = _cpu_baseline(args.cpu_members, args.cpu_nsteps)

    # kernels of ours per integration: init; output; seed; adjoint of the init;
    # stored states: a coefficient kernel + (Legendre, grid) per step forward, a
    # coefficient kernel + (grid adjoint, Legendre adjoint) per step backward;
    # checkpoints: a coefficient kernel per window both ways and, backward, the
    # 2 recompute kernels per step as well
    # (with concurrent groups every per-step kernel runs once per group)
    if store_fast == "all":
        launches = 4 + ng * ((1 + 2 * T_BENCH) + (1 + 2 * T_BENCH))
    else:
        nwin = -(-T_BENCH // CKPT)
        launches = 4 + ng * ((nwin + 2 * T_BENCH) + (nwin + 4 * T_BENCH))
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * t_max, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 state/pointwise, f32 Legendre (fast path); f64 plain path",
        "data": "synthetic (seeded forced ensemble: taurad, taudrag log-uniform [1e4,1e6] s, DPhieq U[1e5,4e6], Phi noise 1e-3*Phibar at n<=10)",
        "config": {"workload": (f"forced ensemble fwd+adjoint, M=42 (64x128), B={B} members per GPU, {T_BENCH} steps, "
                                + ("all states stored (no recomputation)" if store_fast == "all"
                                   else f"checkpoint every {CKPT} (windows recomputed)")),
                   "members_per_gpu": B, "steps_per_member": T_BENCH,
                   "ckpt_every": CKPT if store_fast != "all" else None,
                   "adjoint_states": store_fast,
                   "schedule": (f"{ng} groups of {'/'.join(str(b) for b in _group_sizes(B, ng))} members, "
                                "one stream each (concurrent)") if ng > 1 else "all members in each launch",
                   "l2": "integration touches >= 9 GB (stored states or checkpoints + window slots) > L2 (126 MB); 512 MB L2 flush write between timed steps"},
        "e2e": dropin_e2e if dropin_e2e is not None else {
            "value": round(job_throughput(world, B, T_BENCH, e2e_t), 1), "unit": UNIT,
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "ms_per_step": round(1e3 * e2e_t, 3)},
        "e2e_engine_api": {"value": round(job_throughput(world, B, T_BENCH, e2e_t), 1), "unit": UNIT,
                           "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                           "ms_per_step": round(1e3 * e2e_t, 3),
                           "api": "my_swampe_gb300.adjoint.integrate on an Engine of two concurrent groups"},
        "roofline": roofline,
        "fp64_plain_gpu": fp64,
        "dropin_forward": dropin,
        "mixed_truncations": mixed,
        "emission_stage": emission,
        "cpu_baseline": cpu,
        "gpu_launches": launches * args.steps,
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# The reference's published regime for its forward-scan numbers (paper/speed_benchmark.md:14-19):
# M=42, dt=120 s, Phibar=3e5, omega=3.2e-5, a=8.2e7, taurad=36000 s, taudrag=21600 s,
# DPhieq=1e6 (B=1) or swept 5e5..2e6 (batched), K6=1.24e33, forced, modified Euler, 7,199 steps;
# published on an A100 in FP64 (member-steps/s): B=1 6,241, B=64 58,414.
_PUBLISHED_A100 = {1: 6241.0, 64: 58414.0}


def _dropin_leg(reps=2):
    """Forward throughput through the drop-in API (run_model_scan_final, analytic
    rest-state initial condition, no history) in the reference's published
    regime, at B=1 and B=64, FP64 and fast; the first call of each shape (plan
    build, geometry, graph capture) is reported separately from warm calls."""
    import numpy as np
    import torch

    from my_swampe_gb300 import run_model_scan_final

    kw = dict(M=42, dt=120.0, tmax=2 + 7199, Phibar=3.0e5, omega=3.2e-5, a=8.2e7, taurad=36000.0, taudrag=21600.0,
              K6=1.24e33)
    out = {}
    for B in (1, 64):
        dp = 1.0e6 if B == 1 else [float(x) for x in np.linspace(5.0e5, 2.0e6, B)]
        for prec in ("fp64", "fast"):
            def call():
                r = run_model_scan_final(**kw, DPhieq=dp, precision=prec)
                return r["last_state"].Phi_curr
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            phi = call()
            torch.cuda.synchronize()
            cold = time.perf_counter() - t0
            ts = []
            for _ in range(reps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                phi = call()
                torch.cuda.synchronize()
                ts.append(time.perf_counter() - t0)
            warm = float(np.median(ts))
            out[f"B{B}_{prec}"] = {"member_steps_per_s": round(B * 7199 / warm, 1),
                                   "first_call_member_steps_per_s": round(B * 7199 / cold, 1),
                                   "s_per_call": round(warm, 4), "finite": bool(torch.isfinite(phi).all())}
    out["reference_A100_fp64_published"] = {f"B{k}": v for k, v in _PUBLISHED_A100.items()}
    out["note"] = ("wall clock per run_model_scan_final call (host launch to result on the device), forward only, "
                   "7,199 steps; the A100 rows are the reference's published JAX FP64 numbers on other hardware, "
                   "context rather than a like-for-like ratio")
    return out


def _mixed_leg(steps=2):
    """The mixed-truncation ensemble (64 members at M=42, 32 at M=63, 8 at M=106,
    dt 30 / 20 / 12 s, forced, parameters sampled per member) as one plan:
    forward + adjoint over 1440 steps in the fast precision (tensor-core
    Legendre kernels where the truncation has them), its rate, and the error
    of its forward after 1440 steps against the FP64 plan, per group."""
    import numpy as np
    import torch

    from my_swampe_gb300 import workloads
    from my_swampe_gb300.adjoint import Integration
    from my_swampe_gb300.engine import Engine, RunFlagsC

    spec = [(42, 64, 30.0), (63, 32, 20.0), (106, 8, 12.0)]
    flags = RunFlagsC()
    outs, rate, tc_groups = {}, None, None
    for prec in ("fast", "fp64"):
        eng = Engine([(M, B) for M, B, _ in spec], prec, concurrent=True, autotune=True)
        ics = []
        for g, (M, B, dt) in enumerate(spec):
            wl = workloads.forced_ensemble(eng, g=g, seed=500 + 1000 * g, dt=dt)
            workloads.apply_params(eng, g, wl["params"])
            ics.append(wl["ics"].to(eng.rdtype))
        if prec == "fast":
            tc_groups = eng.tensor_core_groups
            integ = Integration(eng, flags, t0=2, nsteps=T_BENCH, ckpt_every=CKPT)

            def step():
                o = integ.run_forward(ics)
                d = [torch.zeros_like(x) for x in o]
                for x, dx in zip(o, d):
                    dx[2] = x[2] / x[2].numel()
                integ.run_backward(d)

            times = _time_steps(step, steps, 1, lambda: None)
            rate = sum(B for _, B, _ in spec) * T_BENCH / float(np.mean(times))
            store = integ.store
            integ.release()
        eng.init_state(ics, flags)
        eng.forward(flags, t0=2, nsteps=50)
        early = [x.double() for x in eng.output_physical(flags)]
        eng.forward(flags, t0=52, nsteps=T_BENCH - 50)
        eng.check_device_status()
        outs[prec] = (early, [x.double() for x in eng.output_physical(flags)])
        del eng
        torch.cuda.empty_cache()
    err = {}
    for g, (M, B, _) in enumerate(spec):
        # the reference's FP64 algorithm overflows at M=106 in this regime (its damaged
        # basis amplifies modes m = 80..89 on every full re-projection): compared after 50 steps
        late_ok = bool(torch.isfinite(outs["fp64"][1][g]).all())
        at, nst = (1, T_BENCH) if late_ok else (0, 50)
        e = {"after_steps": nst, "fast_finite_after_1440": bool(torch.isfinite(outs["fast"][1][g]).all())}
        for k, name in enumerate(("eta", "delta", "Phi")):
            ref = outs["fp64"][at][g][k]
            dif = outs["fast"][at][g][k] - ref
            e[name] = {"rel_l2": float(torch.linalg.vector_norm(dif) / torch.linalg.vector_norm(ref)),
                       "max_abs": float(dif.abs().max())}
        err[f"M{M}"] = e
    return {"workload": "64 @ M=42 + 32 @ M=63 + 8 @ M=106, forced, 1440 steps, fwd+adjoint, fast precision, "
                        "one plan (groups concurrent)",
            "member_steps_per_s": round(rate, 1), "adjoint_states": store, "tensor_core_groups": tc_groups,
            "error_fast_vs_fp64": err}


def _fp64_peak_tflops(clocks):
    """GB300's FP64 (non-tensor) rate: 2 DFMA per cycle per SM at the sampled SM clock."""
    import torch

    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    return nsm * 2 * 2 * mhz * 1e6 / 1e12


def _emission_leg(B=256, ydeg=10, ntimes=200, reps=20):
    """The retrieval's emission stage on B terminal Phi fields (M = 42 grid):
    Phi -> T -> intensity -> ydeg-10 Ylm coefficients -> phase curve, FP64.
    The projector and the light-curve design matrix are seeded random
    matrices of the right shapes (the kernels' cost does not depend on their
    values)."""
    import numpy as np
    import torch

    from my_swampe_gb300 import emission as em

    J, I = 64, 128
    dev = torch.device("cuda")
    gen = torch.Generator(device=dev).manual_seed(42)
    ncoef = (ydeg + 1) ** 2
    lat = torch.linspace(-1.5, 1.5, J, dtype=torch.float64, device=dev)[:, None]
    lon = torch.linspace(-np.pi, np.pi, I + 1, dtype=torch.float64, device=dev)[None, :I]
    phi = (4e4 * torch.cos(lon) * torch.cos(lat))[None] * (1 + torch.rand((B, 1, 1), generator=gen, device=dev,
                                                                          dtype=torch.float64))
    P = torch.randn((ncoef, J * I), generator=gen, device=dev, dtype=torch.float64) / (J * I)
    A = torch.randn((ntimes, ncoef), generator=gen, device=dev, dtype=torch.float64)
    w = torch.cos(lat[:, 0]) * (np.pi / J)
    amp = torch.full((B,), 1500e-6, dtype=torch.float64, device=dev)
    cfg = em.EmissionConfig()

    def call():
        y = em.emission_coefficients(phi, 4e5, P, w, cfg)
        return em.phase_curve(y, A, amp)

    lc = call()
    assert bool(torch.isfinite(lc).all())
    times = _time_steps(call, reps, 3, lambda: None)
    t = float(np.median(times))
    alg = (B * J * I + ncoef * J * I) * 8  # each Phi field and the projector read once
    return {"workload": f"B={B} terminal Phi fields (M=42 grid) -> T -> T^4 -> ydeg={ydeg} coefficients "
                        f"({ncoef}) -> phase curve at {ntimes} times, FP64",
            "ms_per_call": round(1e3 * t, 4), "members_per_s": round(B / t, 1),
            "algorithmic_gbs": round(alg / t / 1e9, 1), "launches_per_call": 4}


def _cpu_baseline(members, nsteps):
    """The oracle (reference algorithm restated) with torch autograd on the host
    cores: forward + reverse mode over `nsteps` steps for `members` members."""
    import numpy as np
    import torch

    from oracle import swampe_oracle as o

    cores = torch.get_num_threads()
    xp = o.torch_backend()
    geo = o.cached_geometry(M_BENCH)
    J, I = geo["J"], geo["I"]
    rng = np.random.default_rng(7)
    mu = geo["mus"][:, None]
    t_total = 0.0
    for b in range(members):
        tr = torch.tensor(10.0 ** rng.uniform(4, 6), dtype=torch.float64, requires_grad=True)
        td = torch.tensor(10.0 ** rng.uniform(4, 6), dtype=torch.float64, requires_grad=True)
        dp = torch.tensor(rng.uniform(1e5, 4e6), dtype=torch.float64, requires_grad=True)
        pb = torch.tensor(4.0e6, dtype=torch.float64, requires_grad=True)
        Phi0 = torch.tensor(4e3 * rng.standard_normal((J, I)) * 0.1, requires_grad=True)
        eta0 = torch.tensor(2 * 3.2e-5 * mu * np.ones((1, I)), requires_grad=True)
        z = torch.zeros((J, I), dtype=torch.float64)
        t0 = time.perf_counter()
        r = o.run_model_scan_final(xp, M=M_BENCH, dt=30.0, tmax=2 + nsteps, Phibar=pb, omega=3.2e-5, a=8.2e7,
                                   taurad=tr, taudrag=td, DPhieq=dp, eta0_init=eta0, delta0_init=z,
                                   Phi0_init=Phi0, U0_init=z, V0_init=z)
        loss = torch.mean(r["last_state"]["Phi_curr"] ** 2)
        loss.backward()
        t_total += time.perf_counter() - t0
    v = members * nsteps / t_total
    return {"value": round(v, 2), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{members} member(s) x {nsteps} steps fwd+adjoint (torch autograd through the oracle, FP64), M=42"}


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np

    vals = []
    for _ in range(args.warmup):
        _cpu_baseline(1, args.ref_nsteps)
    for _ in range(args.steps):
        vals.append(_cpu_baseline(1, args.ref_nsteps)["value"])
    import torch

    v = float(np.mean(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 2), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * args.ref_nsteps / v, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded forced member, Phi noise), same regime as our arm",
        "config": {"workload": "forced ensemble fwd+adjoint, M=42 (64x128), 1 member x "
                               f"{args.ref_nsteps} steps per timed step (bounded sample of the B=256 x 1440 workload)"},
        "cpu_baseline": {"value": round(v, 2), "unit": UNIT, "cores": torch.get_num_threads(), "kind": "port",
                         "sample": f"1 member x {args.ref_nsteps} steps fwd+adjoint per step; JAX (the reference's "
                                   "runtime) is not installable here, so its algorithm runs as the oracle restatement "
                                   "with torch autograd"},
        "e2e": {"value": round(v, 2), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_profile(args):
    """Small cases of the bench workload for ncu (no timing).

    --profile-case window: one checkpoint window, i.e. init, K forward steps
        (checkpointed), then the window adjoint (K recompute steps + K adjoint
        steps): the kernel mix of the timed bench, for the launch list.
    --profile-case steps: init, 4 forward steps, 3 adjoint steps, each launched
        on its own (no graphs): a handful of launches of every step kernel, for
        full captures (launch order: grid INIT, then per forward step Legendre +
        grid STEP, then per adjoint step grid ADJ_STEP + Legendre adjoint).
    --profile-case sweep: init, 4 forward steps with every state kept, then the
        adjoint sweep over them (its steps after the first skip the zero
        columns, as inside the bench's sweeps).
    --profile-case emission: the emission-stage leg once (B members, FP64)."""
    import torch

    torch.cuda.set_device(0)
    from __graft_entry__ import build

    build()
    if args.profile_case == "emission":
        r = _emission_leg(B=args.B, reps=1)
        print(json.dumps({"profile": "emission", "B": args.B, "ok": True, "ms_per_call": r["ms_per_call"]}))
        return
    from my_swampe_gb300.adjoint import Integration

    # no autotuning here: its timing launches would come before the profiled ones
    eng, wl, flags, _, ics = _setup(args.profile, args.B, ngroups=1, M=args.profile_M, autotune=False)
    if args.profile_case == "sweep":
        eng.init_state(ics, flags)
        gd = eng.groups[0]
        states = [torch.empty((5,) + tuple(gd["fourier"].shape), dtype=eng.cdtype, device=eng.device)]
        eng.forward_stored(flags, t0=2, nsteps=4, states=states)
        lam, lamy, grad = eng.new_adjoint_buffers()
        lam[0].copy_(torch.randn_like(lam[0]))
        eng.adjoint_stored(flags, states, lam, lamy, grad, t0=2, nsteps=4)
        torch.cuda.synchronize()
        eng.check_device_status()
        print(json.dumps({"profile": args.profile, "case": "sweep", "M": args.profile_M, "B": args.B,
                          "tensor_core_groups": eng.tensor_core_groups, "ok": True}))
        return
    if args.profile_case == "steps":
        eng.init_state(ics, flags)
        eng.forward(flags, t0=2, nsteps=3)
        four_in = [eng.groups[0]["fourier"].clone()]
        eng.forward(flags, t0=5, nsteps=1)
        four_out = [eng.groups[0]["fourier"]]
        lam, lamy, grad = eng.new_adjoint_buffers()
        lam[0].copy_(torch.randn_like(lam[0]))
        for _ in range(3):
            eng.adjoint_step(flags, four_in, four_out, lam, lamy, grad, t=6)
        torch.cuda.synchronize()
        eng.check_device_status()
        print(json.dumps({"profile": args.profile, "case": "steps", "M": args.profile_M, "B": args.B,
                          "tensor_core_groups": eng.tensor_core_groups, "ok": True}))
        return
    integ = Integration(eng, flags, t0=2, nsteps=CKPT, ckpt_every=CKPT)
    out = integ.run_forward(ics)[0]
    d = torch.zeros_like(out)
    d[2] = out[2] / out[2].numel()
    integ.run_backward([d])
    torch.cuda.synchronize()
    print(json.dumps({"profile": args.profile, "B": args.B, "steps": CKPT, "ok": True}))


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--B", type=int, default=B_BENCH)
    ap.add_argument("--groups", type=int, default=2, choices=(1, 2, 3, 4),
                    help="split the ensemble into this many concurrent groups (one stream each)")
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-dropin", action="store_true", help="skip the drop-in API forward leg")
    ap.add_argument("--skip-mixed", action="store_true", help="skip the mixed-truncation leg")
    ap.add_argument("--skip-emission", action="store_true", help="skip the emission-stage leg")
    ap.add_argument("--cpu-members", type=int, default=1)
    ap.add_argument("--cpu-nsteps", type=int, default=40)
    ap.add_argument("--ref-nsteps", type=int, default=20)
    ap.add_argument("--profile", choices=("fast", "fp64"), default=None,
                    help="run a small case of the workload (for ncu) instead of timing")
    ap.add_argument("--profile-case", choices=("window", "steps", "sweep", "emission"), default="window")
    ap.add_argument("--profile-M", type=int, choices=(42, 63, 106), default=M_BENCH,
                    help="truncation of the profiled case")
    ap.add_argument("--store", choices=("auto", "all", "checkpoint"), default="auto",
                    help="how the adjoint gets its primal states (Integration store policy)")
    args = ap.parse_args()
    if args.profile:
        run_profile(args)
        return
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
