"""Benchmark: batched friction-contact QP solves per second on GB300.

Workload (one step): 4096 independent friction-contact QPs, c ~ U{4..64} contacts each
(n = 3c forces, m = 4c cone rows: R^c_+ x c Q^3), solved to the 1e-8 relative gap by one
batched mixed-precision (FP32 factor, FP64 refinement) launch sequence. Synthetic, seeded data
of the reference's contact-problem shape; cold starts (warm_start off) so every step repeats
the full solve. Inputs stay resident in HBM; the L2 is flushed (256 MB write) between timed steps.

  value  -- solves/s of the device-resident batch (CUDA events on the solver's stream)
  e2e    -- the same through the C-ABI with pinned HOST buffers: H2D of the step's values,
            solve, D2H of x, s, z inside the timed region
  cpu_baseline -- the FP64 CPU restatement of the reference (oracle, "port") on the host cores,
            one instance per thread, on a bounded sample
  plain_gpu -- the plain per-instance GPU form (FP64 factor, one launch per solve)

`--impl reference` times the reference's CPU path (the oracle port; the reference itself cannot
be built here) on the same workload with every host thread.
Multi-GPU: one process per GPU (torchrun); each rank solves its own 4096-instance batch (weak
scaling, no data-path collective); the reported time is the max over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "QP solves/s at 1e-8 rel. gap: batched mixed-prec vs plain GPU vs host CPU; fwd+bwd µs"
COUNT = 4096


def workload(count):
    return (f"batched friction-contact QPs: {count} instances, c~U{{4..64}}, n=3c, cones R^c_+ x c Q^3, "
            "mixed FP32/FP64")


WORKLOAD = workload(COUNT)


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def run_gb300(args, rank, world, local_rank):
    import torch

    from conicxx_gb300 import BatchSolver, Solver, default_settings, generators
    from conicxx_gb300._abi import INFO_DTYPE

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    count = args.count
    qps = generators.contact_batch(count, base_seed=rank * count)
    st = default_settings(precision=1, warm_start=0)
    t0 = time.perf_counter()
    B = BatchSolver(qps, settings=st)
    setup_s = time.perf_counter() - t0
    tune_report = B.autotune(trials=2) if args.autotune else None
    Px, q, Ax, b = B.concat_values()
    dvals = [torch.from_numpy(v).to(dev) for v in (Px, q, Ax, b)]
    dx = torch.empty(B.n_total, dtype=torch.float64, device=dev)
    ds = torch.empty(B.m_total, dtype=torch.float64, device=dev)
    dz = torch.empty(B.m_total, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream

    def solve_step():
        if args.entry == "noalloc":
            B.solve_device_noalloc(int(dx.data_ptr()), int(ds.data_ptr()), int(dz.data_ptr()), sp)
        else:
            B.solve_device(int(dx.data_ptr()), int(ds.data_ptr()), int(dz.data_ptr()), sp)

    def step(ev=None):
        B.update_values_device(*(int(t.data_ptr()) for t in dvals), sp)
        if ev is not None:
            ev.record(stream)
        solve_step()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    torch.cuda.synchronize()
    launches_per_step = B.last_launches()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    sampler = ClockSampler(local_rank)
    sampler.start()
    evs = [tuple(torch.cuda.Event(enable_timing=True) for _ in range(3)) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.fill_(i & 0xFF)  # evict the L2 between timed steps
            evs[i][0].record(stream)
            step(evs[i][1])
            evs[i][2].record(stream)
    torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - w0
    clocks = sampler.stop()
    step_ms = np.array([a.elapsed_time(c_) for a, _, c_ in evs])
    ipm_ms = float(np.mean([b_.elapsed_time(c_) for _, b_, c_ in evs]))
    ms_local = float(step_ms.mean())
    ms = ms_local
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([ms_local], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    infos = np.zeros(count, dtype=INFO_DTYPE)
    if args.entry == "noalloc":
        B.solve_device_noalloc(int(dx.data_ptr()), int(ds.data_ptr()), int(dz.data_ptr()), sp, infos)
    else:
        B.solve_device(int(dx.data_ptr()), int(ds.data_ptr()), int(dz.data_ptr()), sp, infos)
    solved_frac = float(np.mean(infos["status"] == 1))
    statuses = {int(k): int(v) for k, v in zip(*np.unique(infos["status"], return_counts=True))}

    result = {}
    if rank == 0 and args.legs == "main":
        hbm_peak, peak_kind = peaks()
        achieved = B.algorithmic_bytes() / (ipm_ms * 1e-3) / 1e9
        result = dict(roofline={"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                                "frac": achieved / hbm_peak, "traffic": None, "peak_kind": peak_kind,
                                "ipm_ms": ipm_ms})
    elif rank == 0:
        # ---- e2e through the C-ABI with pinned host buffers ----
        pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
        hvals = [pin(v) for v in (Px, q, Ax, b)]
        hx, hs, hz = (pin(np.zeros(k)) for k in (B.n_total, B.m_total, B.m_total))
        from conicxx_gb300._abi import dptr
        from conicxx_gb300._lib import check, lib

        L = lib()

        def e2e_step():
            check(L.cxg_batch_update_values(B._h, *(dptr(v) for v in hvals)), "update")
            check(L.cxg_batch_solve(B._h, dptr(hx), dptr(hs), dptr(hz), None), "solve")

        for _ in range(max(1, args.warmup // 2)):
            e2e_step()
        e0 = time.perf_counter()
        e2e_steps = max(2, args.steps)
        for _ in range(e2e_steps):
            e2e_step()
        e2e_s = (time.perf_counter() - e0) / e2e_steps
        h2d = 8 * (B.nnzP + B.n_total + B.nnzA + B.m_total)
        d2h = 8 * (B.n_total + 2 * B.m_total)
        # ---- plain per-instance GPU form (FP64 factor, one solve per launch) ----
        plain_n = args.plain_instances
        sub = qps[:plain_n]
        solvers = []
        for qp in sub:
            S = Solver()
            assert S.setup(qp, warm_start=0)
            solvers.append(S)
        solvers[0].solve()
        p0 = time.perf_counter()
        for S in solvers:
            S.solve()
        plain_s = time.perf_counter() - p0
        plain_rate = plain_n / plain_s
        # ---- differentiable layer: 1024 instances n=100, m=150 (Zero^10 x R^100_+ x 10 Q^4),
        # forward alone vs forward + adjoint (dL/dq, dL/db, dL/dP, dL/dA for L = 1/2|x - t|^2) ----
        dqps = generators.config3_batch(1024)
        DB = BatchSolver(dqps, settings=default_settings(precision=1, warm_start=0, differentiable=1))
        dv = [torch.from_numpy(v).to(dev) for v in DB.concat_values()]
        dxx = torch.empty(DB.n_total, dtype=torch.float64, device=dev)
        dss = torch.empty(DB.m_total, dtype=torch.float64, device=dev)
        dzz = torch.empty(DB.m_total, dtype=torch.float64, device=dev)
        tgt = torch.from_numpy(np.concatenate([generators.x_target(i, q_.n) for i, q_ in enumerate(dqps)])).to(dev)
        gq = torch.empty(DB.n_total, dtype=torch.float64, device=dev)
        gbb = torch.empty(DB.m_total, dtype=torch.float64, device=dev)
        gP = torch.empty(DB.nnzP, dtype=torch.float64, device=dev)
        gA = torch.empty(DB.nnzA, dtype=torch.float64, device=dev)

        def fwd():
            DB.update_values_device(*(int(t.data_ptr()) for t in dv), sp)
            DB.solve_device(int(dxx.data_ptr()), int(dss.data_ptr()), int(dzz.data_ptr()), sp)

        def bwd():
            gx = dxx - tgt
            DB.backward_device(int(gx.data_ptr()), int(gq.data_ptr()), int(gbb.data_ptr()), int(gP.data_ptr()),
                               int(gA.data_ptr()), sp)

        with torch.cuda.stream(stream):
            for _ in range(2):
                fwd()
                bwd()
            torch.cuda.synchronize()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            fw, fb = [], []
            for _ in range(max(2, args.steps)):
                e[0].record(stream)
                fwd()
                e[1].record(stream)
                bwd()
                e[2].record(stream)
                torch.cuda.synchronize()
                fw.append(e[0].elapsed_time(e[1]))
                fb.append(e[0].elapsed_time(e[2]))
        fwd_bwd = {"instances": 1024, "workload": "n=100, m=150, Zero^10 x R^100_+ x 10 Q^4, L=1/2|x-t|^2",
                   "fwd_us": 1e3 * float(np.median(fw)), "fwd_bwd_us": 1e3 * float(np.median(fb)),
                   "ratio": float(np.median(fb) / np.median(fw))}
        # ---- CPU baseline: oracle restatement on the host cores ----
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc

        orc.build()
        # ---- one instance of n=200, m=300 (Zero^20 x R^160_+ x 40 Q^3): the plain GPU form in
        # FP64 against the oracle on one host core ----
        qp0 = generators.config0_qp(0)
        S0 = Solver()
        assert S0.setup(qp0, warm_start=0)
        S0.solve()
        g_ms = []
        for _ in range(5):
            t0_ = time.perf_counter()
            sol0 = S0.solve()
            g_ms.append(1e3 * (time.perf_counter() - t0_))
        S0m = Solver()
        assert S0m.setup(qp0, warm_start=0, precision=1)
        S0m.solve()
        m_ms = []
        for _ in range(5):
            t0_ = time.perf_counter()
            sol0m = S0m.solve()
            m_ms.append(1e3 * (time.perf_counter() - t0_))
        O0 = orc.OracleSolver()
        assert O0.setup(qp0, warm_start=0)
        O0.solve()
        c_ms = []
        for _ in range(5):
            t0_ = time.perf_counter()
            _, _, _, oi0 = O0.solve()
            c_ms.append(1e3 * (time.perf_counter() - t0_))
        single = {"workload": "n=200, m=300, Zero^20 x R^160_+ x 40 Q^3, one instance, FP64",
                  "gpu_ms": float(np.median(g_ms)), "gpu_mixed_ms": float(np.median(m_ms)),
                  "cpu_1core_ms": float(np.median(c_ms)), "iterations_gpu_mixed": int(sol0m.info["iterations"]),
                  "iterations_gpu": int(sol0.info["iterations"]), "iterations_cpu": int(oi0["iterations"]),
                  "status_gpu": int(sol0.status), "status_cpu": int(oi0["status"])}
        large = large_instance_leg(orc, args.large_fp64, args.large_full)
        # ---- the same batch with the FP64 factor (configuration 1 names FP64 and mixed) ----
        B64 = BatchSolver(qps, settings=default_settings(precision=0, warm_start=0))
        dx64 = torch.empty_like(dx)
        ds64 = torch.empty_like(ds)
        dz64 = torch.empty_like(dz)

        def step64():
            B64.update_values_device(*(int(t.data_ptr()) for t in dvals), sp)
            B64.solve_device(int(dx64.data_ptr()), int(ds64.data_ptr()), int(dz64.data_ptr()), sp)

        with torch.cuda.stream(stream):
            step64()
            torch.cuda.synchronize()
            e64 = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            t64 = []
            for i in range(2):
                flush.fill_(i & 0xFF)
                e64[0].record(stream)
                step64()
                e64[1].record(stream)
                torch.cuda.synchronize()
                t64.append(e64[0].elapsed_time(e64[1]))
        infos64 = np.zeros(count, dtype=INFO_DTYPE)
        B64.solve_device(int(dx64.data_ptr()), int(ds64.data_ptr()), int(dz64.data_ptr()), sp, infos64)
        torch.cuda.synchronize()
        fp64_batch = {"value": count / (1e-3 * float(np.median(t64))), "unit": "solves/s",
                      "ms_per_step": float(np.median(t64)),
                      "statuses": {int(k): int(v) for k, v in zip(*np.unique(infos64["status"], return_counts=True))}}
        ncpu = os.cpu_count() or 1
        sample = qps[:args.cpu_sample]
        cpu_wall, cpu_st, cpu_it, ox, os_, oz = orc.batch_solve_x(sample, ncpu, warm_start=0)
        cpu_rate = len(sample) / cpu_wall
        # ---- per-instance error against the FP64 oracle on that sample, both precisions ----
        errors = {"sample": f"first {len(sample)} instances",
                  "metric": "max |v_gpu - v_oracle| / max(1, max |v_oracle|) per instance, v = x, s, z"}
        for name, inf_, tx, ts, tz in (("mixed", infos, dx, ds, dz), ("fp64", infos64, dx64, ds64, dz64)):
            gx, gs, gz = (t.cpu().numpy() for t in (tx, ts, tz))
            errors[name] = parity_summary(sample, B, inf_[:len(sample)], cpu_st, cpu_it, (gx, gs, gz), (ox, os_, oz))
        # the reference against itself: the same sample with q moved at the last bit (oracle.perturb_q),
        # the scale of rounding-level differences on this family
        _, pst, pit, px, ps_, pz = orc.batch_solve_x([orc.perturb_q(q_, 1 + i) for i, q_ in enumerate(sample)], ncpu,
                                                     warm_start=0)
        pinf = np.zeros(len(sample), dtype=INFO_DTYPE)
        pinf["status"], pinf["iterations"] = pst, pit
        errors["oracle_q_last_bit"] = parity_summary(sample, B, pinf, cpu_st, cpu_it, (px, ps_, pz), (ox, os_, oz))
        # ---- roofline of the IPM launch set (one persistent launch per size bucket, run
        # concurrently; timed by CUDA events around the solve on the launching stream) ----
        hbm_peak, peak_kind = peaks()
        algo_bytes = B.algorithmic_bytes()
        achieved = algo_bytes / (ipm_ms * 1e-3) / 1e9
        # compute bound: the root LDL' (nr^3/6 multiply-adds per factorisation) and its triangular
        # solves (nr^2 per solve pair; 3 solves per iteration plus the refinement steps) on the
        # FP32 CUDA cores, per instance from its iterations and refinement counts
        nr = np.array([qp_.n + qp_.zero for qp_ in qps], dtype=np.float64)
        it = infos["iterations"].astype(np.float64)
        fma = float(np.sum(it * nr ** 3 / 6.0 + (3.0 * it + infos["refine_steps"]) * nr ** 2))
        tflops = 2.0 * fma / (ipm_ms * 1e-3) / 1e12
        fp32_peak = 2.0 * 152 * 128 * 2.07e9 / 1e12
        traffic, fp64_pipe = None, None
        tp = os.path.join(ROOT, "profiles", "ipm_kernel_traffic.json")
        if os.path.exists(tp):
            with open(tp) as f:
                tj = json.load(f)
            # DRAM bytes of the launch set scale with the number of instances
            traffic = tj["dram_bytes_per_step"] * count / tj["instances"]
            fp64_pipe = tj.get("fp64_pipe_active_frac")
        # ---- per-timestep contact-pattern change: a new set-up of 1% and 10% of the instances
        # (cxg_batch_replace: only those planned again, the rest moved on the device) against
        # setting the whole batch up ----
        PB = BatchSolver(qps, settings=default_settings(precision=1, warm_start=1))
        rng_pu = np.random.default_rng(7)
        pattern_update = {"full_setup_s": setup_s, "workload": "contact instances replaced by new contact instances "
                          "(other sizes and patterns), the rest kept with values and warm starts"}
        for pct in (1, 10):
            k = max(1, count * pct // 100)
            idx = rng_pu.choice(count, k, replace=False)
            new = [generators.contact_qp(10_000_000 + 1000 * pct + j) for j in range(k)]
            pattern_update[f"replace_{pct}pct"] = {"instances": int(k), "s": PB.replace(idx, new)}
        del PB
        result = dict(
            pattern_update=pattern_update,
            e2e={"value": count / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            plain_gpu={"value": plain_rate, "unit": "solves/s", "instances": plain_n, "precision": "fp64",
                       "batched_over_plain": (count / (ms * 1e-3)) / plain_rate},
            cpu_baseline={"value": cpu_rate, "unit": "solves/s", "cores": ncpu, "kind": "port",
                          "sample": f"first {len(sample)} of the {count} instances, one instance per thread, "
                                    f"cold start, FP64 oracle restatement of the reference",
                          "solved_fraction": float(np.mean(cpu_st == 1))},
            roofline={"bound": "fp32", "achieved": tflops, "peak": fp32_peak, "unit": "TFLOP/s",
                      "frac": tflops / fp32_peak, "traffic": traffic,
                      "peak_kind": "nominal FP32 CUDA-core rate: 152 SMs x 128 FMA/clock x 2.07 GHz (no measured "
                                   "FP32 figure exists for this pool)",
                      "ipm_ms": ipm_ms, "multiply_adds": fma, "fp64_pipe_active_frac": fp64_pipe,
                      "hbm": {"achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                              "peak_kind": peak_kind, "algorithmic_bytes": algo_bytes},
                      "note": "IPM launch set (one persistent launch per size bucket). Compute: sum over "
                              "instances of iterations x nr^3/6 (root LDL') + (3 x iterations + refinement "
                              "steps) x nr^2 (triangular solves) multiply-adds, 2 flops each; instances that "
                              "hold the double-float factor spend about 12 FP32 operations per such "
                              "multiply-add. HBM: plans + values + solutions + results once; the whole "
                              "problem lives in shared memory and L2 for every iteration, so HBM is not the "
                              "bound. The makespan is set by the slowest instances' serial FP64/double-float "
                              "chains"},
            fp64_batch=fp64_batch,
            parity_vs_oracle=errors,
            fwd_bwd=fwd_bwd,
            single_instance=single,
            large_instance=large,
            setup_s=setup_s,
        )
    if tune_report is not None:
        result["autotune"] = tune_report.strip().splitlines()
    return ms, wall, clocks, launches_per_step, solved_frac, statuses, result


def parity_summary(sample, B, infos, cpu_st, cpu_it, gpu, orc_):
    """Status agreement, iteration differences and per-instance x/s/z errors of the device batch
    against the FP64 oracle on the instances of `sample` (the first len(sample) of batch B)."""
    gx, gs, gz = gpu
    ox, os_, oz = orc_
    st_g = infos["status"].astype(int)
    st_o = np.asarray(cpu_st, int)
    both = (st_g == 1) & (st_o == 1)
    errs = {"x": [], "s": [], "z": []}
    for i, qp in enumerate(sample):
        if not both[i]:
            continue
        # the sample is the batch's first instances, so both concatenations share the offsets
        for key, g, o, off, ln in (("x", gx, ox, B.n_off[i], qp.n), ("s", gs, os_, B.m_off[i], qp.m),
                                   ("z", gz, oz, B.m_off[i], qp.m)):
            ov, gv = o[off:off + ln], g[off:off + ln]
            errs[key].append(float(np.max(np.abs(gv - ov)) / max(1.0, float(np.max(np.abs(ov))))))
    dit = (infos["iterations"].astype(int) - np.asarray(cpu_it, int))[both]
    out = {"status_agree": int(np.sum(st_g == st_o)), "instances": len(sample),
           "status_mismatches": [[i, int(st_g[i]), int(st_o[i])] for i in np.nonzero(st_g != st_o)[0].tolist()],
           "both_solved": int(both.sum()),
           "iterations_equal_frac": float(np.mean(dit == 0)) if dit.size else None,
           "iterations_within_1_frac": float(np.mean(np.abs(dit) <= 1)) if dit.size else None}
    for key, v in errs.items():
        v = np.array(v)
        if v.size:
            out[key] = {"median": float(np.median(v)), "p99": float(np.quantile(v, 0.99)), "max": float(v.max()),
                        "frac_le_1e-6": float(np.mean(v <= 1e-6))}
    return out


def large_instance_leg(orc, fp64_factor=False, groups_full=False):
    """Single large instances on the whole GPU (root spread over every SM), mixed precision:
    - the n=20000, m=30000 sparse QP (root of 22000 rows): the full solve to 1e-8 (status,
      iterations, time, KKT residuals of the returned point), and its first 3 iterations alone
      for the FP32 factor's throughput (tensor-core trailing updates);
    - with fp64_factor, the same instance solved again with the FP64 factor (precision 0), and
      the largest differences of x, s and z between the two runs;
    - the group-lasso SOCP with 1000 groups of 16 (n=17000, 1000 SOC blocks of dimension 17),
      solved to completion; with groups_full, also at 4000 groups (n=68000, a 68000-row root);
    - the sparse QP family at n=1000 (root of 1100 rows) against the oracle on one host core."""
    from conicxx_gb300 import Solver, generators

    out = {}
    qp = generators.large_sparse_qp(0)
    S = Solver()
    assert S.setup(qp, precision=1, warm_start=0, record_timings=1, max_iter=3)
    t0 = time.perf_counter()
    sol = S.solve()
    dt = time.perf_counter() - t0
    inf = sol.info
    nr = qp.n + qp.zero
    per_fact = inf["time_ldlt_s"] / max(1, inf["factor_attempts"])
    clock_hz = 2.07e9
    fp32_peak = 152 * 128 * clock_hz / 1e12  # FP32 FMA/s of the CUDA cores at the maximum SM clock
    tfma = (nr ** 3 / 6) / per_fact / 1e12
    bf16 = None
    mp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(mp):
        with open(mp) as f:
            bf16 = json.load(f).get("bf16_tflops")
    # 3xTF32 on the tensor pipe: TF32 runs at half the dense BF16 rate, three MMAs per product
    tc_ceiling = (bf16 / 2.0 / 2.0 / 3.0) if bf16 else None
    first3 = {
        "iterations_timed": int(inf["iterations"]), "s_per_iteration": dt / max(1, inf["iterations"]),
        "factorisations": int(inf["factor_attempts"]), "fp32_assembly_ldlt_s": per_fact,
        "fp32_ldlt_tfma_s": tfma, "fp32_cuda_core_peak_tfma_s": fp32_peak, "frac_cuda_core": tfma / fp32_peak,
        "tensor_3xtf32_ceiling_tfma_s": tc_ceiling,
        "frac_tensor_3xtf32": (tfma / tc_ceiling) if tc_ceiling else None,
        "dense_solve_s": inf["time_dense_solve_s"], "fp64_fallbacks": int(inf["fp64_fallbacks"])}
    S = Solver()
    assert S.setup(qp, precision=1, warm_start=0, record_timings=1)
    t0 = time.perf_counter()
    sol = S.solve()
    dt = time.perf_counter() - t0
    inf = sol.info
    st_, fe_, sz_ = qp.kkt_residuals(sol.x, sol.s, sol.z)
    out["sparse_qp_n20000"] = {
        "workload": "n=20000, m=30000, Zero^2000 x R^24000_+ x 2000 Q^2, P=M'M+1e-3 I (3 nnz/col), A 8 nnz/row",
        "root_rows": nr, "status": int(sol.status), "iterations": int(inf["iterations"]), "solve_s": dt,
        "s_per_iteration": dt / max(1, inf["iterations"]), "fp64_fallbacks": int(inf["fp64_fallbacks"]),
        "factor_attempts": int(inf["factor_attempts"]), "ldlt_s": inf["time_ldlt_s"],
        "dense_solve_s": inf["time_dense_solve_s"], "max_relres": inf["max_relres"],
        "kkt_residuals": [float(st_), float(fe_), float(sz_)], "first_3_iterations": first3}
    if fp64_factor:
        S64 = Solver()
        assert S64.setup(qp, precision=0, warm_start=0, record_timings=1)
        t0 = time.perf_counter()
        sol64 = S64.solve()
        dt64 = time.perf_counter() - t0
        inf64 = sol64.info
        r64 = qp.kkt_residuals(sol64.x, sol64.s, sol64.z)

        def rdiff(a, b):
            return float(np.max(np.abs(a - b)) / max(1.0, float(np.max(np.abs(b)))))

        out["sparse_qp_n20000"]["fp64_factor"] = {
            "status": int(sol64.status), "iterations": int(inf64["iterations"]), "solve_s": dt64,
            "factor_attempts": int(inf64["factor_attempts"]), "ldlt_s": inf64["time_ldlt_s"],
            "kkt_residuals": [float(v) for v in r64],
            "objective_mixed": float(sol.objective), "objective_fp64": float(sol64.objective),
            "mixed_vs_fp64": {"x": rdiff(sol.x, sol64.x), "s": rdiff(sol.s, sol64.s), "z": rdiff(sol.z, sol64.z),
                              "metric": "max |v_mixed - v_fp64| / max(1, max |v_fp64|)"}}
    for groups in ((1000, 4000) if groups_full else (1000,)):
        qpg = generators.group_lasso_socp(0, groups=groups)
        S = Solver()
        assert S.setup(qpg, precision=1, warm_start=0, record_timings=1)
        t0 = time.perf_counter()
        sol = S.solve()
        dt = time.perf_counter() - t0
        inf = sol.info
        st_, fe_, sz_ = qpg.kkt_residuals(sol.x, sol.s, sol.z)
        out["group_lasso_g%d" % groups] = {
            "workload": "%d groups of 16: n=%d, F %d x %d (12 nnz/row, 64 blocks + 5%% coupling), %d Q^17"
                        % (groups, 17 * groups, 20 * groups, 16 * groups, groups),
            "root_rows": qpg.n + qpg.zero, "solve_s": dt, "status": int(sol.status),
            "iterations": int(inf["iterations"]), "fp64_fallbacks": int(inf["fp64_fallbacks"]),
            "factor_attempts": int(inf["factor_attempts"]), "ldlt_s": inf["time_ldlt_s"],
            "dense_solve_s": inf["time_dense_solve_s"], "kkt_residuals": [float(st_), float(fe_), float(sz_)]}
    qps = generators.large_sparse_qp(0, n=1000, m_zero=100, m_nonneg=1200, n_soc=100)
    times = {}
    for prec in (0, 1):
        S = Solver()
        assert S.setup(qps, precision=prec, warm_start=0)
        S.solve()
        t0 = time.perf_counter()
        sol = S.solve()
        times[prec] = (time.perf_counter() - t0, sol)
    O = orc.OracleSolver()
    assert O.setup(qps, warm_start=0)
    t0 = time.perf_counter()
    xo, _, _, io = O.solve()
    tc = time.perf_counter() - t0
    out["sparse_qp_n1000"] = {
        "workload": "n=1000, m=1500, Zero^100 x R^1200_+ x 100 Q^2 (same family), root of 1100 rows",
        "gpu_fp64_s": times[0][0], "gpu_mixed_s": times[1][0], "cpu_1core_s": tc,
        "status_gpu": int(times[1][1].status), "status_cpu": int(io["status"]),
        "iterations_gpu": int(times[1][1].info["iterations"]), "iterations_cpu": int(io["iterations"]),
        "x_maxdiff_rel": float(np.max(np.abs(times[1][1].x - xo)) / max(1.0, np.max(np.abs(xo))))}
    return out


def ldlt_probe(nr, nx, arith, threads, seed=1, check=False):
    """The dense root LDL' and triangular solve alone (cxg_dense_ldlt) on a seeded quasi-definite
    matrix of the reduced-KKT shape [P, A_Z'; A_Z, -0.5 I]: P = B B'/nx + I (nx x nx), A_Z ~ 0.5
    N(0,1). threads -1 runs the whole-GPU root (every SM); 32..256 the one-CTA root. Returns factor
    and solve time (ns from the device timer, or SM cycles for one CTA), multiply-adds per second,
    the pivot flags and, with check, the relative error against a float64 solve."""
    from conicxx_gb300 import _abi, _lib

    rng = np.random.default_rng(seed)
    B = rng.standard_normal((nx, nx))
    K = np.zeros((nr, nr), order="F")
    K[:nx, :nx] = B @ B.T / nx + np.eye(nx)
    AZ = rng.standard_normal((nr - nx, nx)) * 0.5
    K[nx:, :nx] = AZ
    K[:nx, nx:] = AZ.T
    K[nx:, nx:] = -0.5 * np.eye(nr - nx)
    b = np.random.default_rng(seed + 1).standard_normal(nr)
    D, x = np.zeros(nr), np.zeros(nr)
    cyc = np.zeros(2, np.int64)
    flags = np.zeros(3, np.int32)
    code = {"fp64": 0, "fp32": 1, "df64": 2}[arith]
    rc = _lib.lib().cxg_dense_ldlt(nr, nx, K.ctypes.data, b.ctypes.data, code, threads, _abi.LINSOLVER_QDLDL,
                                   None, D.ctypes.data, x.ctypes.data, cyc.ctypes.data, flags.ctypes.data)
    if rc != _abi.OK:
        raise RuntimeError(_lib.lib().cxg_last_error().decode())
    out = {"probe": "dense root LDL'", "nr": nr, "nx": nx, "arith": arith, "threads": threads,
           "flags": flags.tolist()}
    fma = nr ** 3 / 6.0
    if threads < 0:
        out.update(ldlt_ms=cyc[0] / 1e6, solve_ms=cyc[1] / 1e6, ldlt_fma_per_s=fma / (cyc[0] * 1e-9))
    else:
        out.update(ldlt_cycles=int(cyc[0]), solve_cycles=int(cyc[1]))
    if check:
        xs = np.linalg.solve(K, b)
        out["x_rel_err"] = float(np.linalg.norm(x - xs) / np.linalg.norm(xs))
    return out


def run_reference(args, rank, world):
    """The reference's CPU path: the FP64 oracle restatement (the reference itself cannot be
    built in this environment), all host threads, one instance per thread."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    from conicxx_gb300 import generators

    if rank != 0:
        return None
    orc.build()
    count = args.count
    qps = generators.contact_batch(count)
    ncpu = os.cpu_count() or 1
    sample = min(args.cpu_sample, count)
    rates = []
    for i in range(args.warmup + args.steps):
        lo = (i * sample) % count
        sub = qps[lo:lo + sample]
        wall, st, _ = orc.batch_solve(sub, ncpu, warm_start=0)
        if i >= args.warmup:
            rates.append(len(sub) / wall)
    value = float(np.mean(rates))
    return {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sample / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded contact generator)",
        "config": {"workload": workload(count), "count_per_gpu": count, "sample_per_step": sample,
                   "parallelism": "host threads", "warm_start": False},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": ncpu, "kind": "port",
                         "sample": f"{sample} instances per step, one instance per thread, cold start"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=1024)
    ap.add_argument("--plain-instances", type=int, default=16)
    ap.add_argument("--count", type=int, default=COUNT, help="contact instances per GPU")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="skip cxg_batch_autotune (size-bucket edges and threads per bucket picked by timing whole "
                         "solves before the timed steps; on by default)")
    ap.add_argument("--entry", default="graph", choices=["graph", "noalloc"],
                    help="graph: the captured concurrent-bucket solve (default); noalloc: the allocation-free "
                         "entry point (direct launches, buckets in sequence)")
    ap.add_argument("--legs", default="all", choices=["all", "main", "large"],
                    help="main: only the device-resident batched timing (profiling runs); large: only the "
                         "single large instances (configurations 2 and 4) on the whole GPU")
    ap.add_argument("--large-fp64", action="store_true",
                    help="large instances: also solve configuration 2 with the FP64 factor and compare")
    ap.add_argument("--large-full", action="store_true",
                    help="large instances: also solve configuration 4 at full size (4000 groups)")
    ap.add_argument("--probe-ldlt", type=int, default=0, metavar="NR",
                    help="instead of the benchmark: time the dense root LDL' alone on an NR-row matrix")
    ap.add_argument("--probe-arith", default="fp32", choices=["fp64", "fp32", "df64"])
    ap.add_argument("--probe-threads", type=int, default=-1, help="-1: whole-GPU root; 32..256: one CTA")
    ap.add_argument("--probe-repeat", type=int, default=1)
    ap.add_argument("--probe-check", action="store_true")
    args = ap.parse_args()
    rank, world, local_rank = dist_env()
    if args.probe_ldlt:
        if not os.path.exists(os.path.join(ROOT, "conicxx_gb300", "_build", "libconicxx_gb300.so")):
            import __graft_entry__

            __graft_entry__.build()
        nr = args.probe_ldlt
        for _ in range(args.probe_repeat):
            print(json.dumps(ldlt_probe(nr, max(1, nr - 256), args.probe_arith, args.probe_threads,
                                        check=args.probe_check)), flush=True)
        return
    if args.legs == "large":
        if not os.path.exists(os.path.join(ROOT, "conicxx_gb300", "_build", "libconicxx_gb300.so")):
            import __graft_entry__

            __graft_entry__.build()
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc

        orc.build()
        print(json.dumps({"large_instance": large_instance_leg(orc, args.large_fp64, args.large_full)}), flush=True)
        return
    if args.impl == "reference":
        out = run_reference(args, rank, world)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    if not os.path.exists(os.path.join(ROOT, "conicxx_gb300", "_build", "libconicxx_gb300.so")):
        import __graft_entry__

        __graft_entry__.build()
    ms, wall, clocks, launches, solved_frac, statuses, extra = run_gb300(args, rank, world, local_rank)
    if rank == 0:
        out = {
            "metric": METRIC, "value": world * args.count / (ms * 1e-3), "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "mixed fp32-factor/fp64",
            "data": "synthetic (seeded contact generator)",
            "config": {"workload": workload(args.count), "count_per_gpu": args.count, "entry": args.entry,
                       "autotuned": bool(args.autotune),
                       "parallelism": f"instances x{world}",
                       "l2": "flushed between timed steps (256 MB device write outside the step events)",
                       "solved_fraction": solved_frac, "statuses": statuses, "warm_start": False},
            "wall_s_timed_region": wall, "gpu_launches": launches * args.steps, "clocks": clocks,
        }
        out.update(extra)
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
