"""Benchmark of the Fourier intersection-volume hot path on GB300.

Workload (default): the 256-object volume matrix -- 128 icosphere-4 (5,120
triangles, affine-deformed) + 128 boxes, random rotations, centres U[0,8]^3,
k-grid L=64 x Lebedev-1202 (N_k = 76,928).  One step = one cold volume matrix
from device-resident geometry: DoF transform + form factors (5.05e10
triangle x k evaluations) + contraction V = Re(J^H D J).

    python bench.py [--gpus N --steps K --warmup W] [--impl reference] [--precision fp32|bf16x3|tf32x3|fp16x3]

`value`  : triangle x k evaluations per second over the whole job (inputs
           resident in HBM; L2 flushed before every timed step).
`e2e`    : the same metric through the C ABI's host-buffer entry point
           pi_volume_matrix_host (host geometry in, host V out).
Multi-GPU: weak scaling -- every rank evaluates its own seeded 256-object
matrix; no collective on the data path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "tri×k evals/s; vol-matrix/s BF16-TC vs FP32 at 1e-4 rel err; p50/p99 ms"
UNIT = "tri×k evals/s"
SFU_OPS_PER_EVAL = 9      # 3 complex exponentials (6) + 3 reciprocals, reference algorithm count
FP32_FLOPS_PER_EVAL = 40  # reference algorithm count (FMA = 2)
SFU_PER_SM_PER_CLK = 16   # nominal MUFU results per SM per clock
FP32_FLOPS_PER_SM_PER_CLK = 256


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--precision", default="auto", choices=["auto", "fp32", "bf16x3", "tf32x3", "fp16x3"])
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-serve", action="store_true", help="skip the serving measurements")
    p.add_argument("--no-configs", action="store_true", help="skip the other workload configurations")
    p.add_argument("--serve-queries", type=int, default=240,
                   help="scene-stream sample size (the stream workload has 10,000 queries; see --stream-full)")
    p.add_argument("--serve-plain-prefix", type=int, default=100,
                   help="queries of the stream timed one at a time on the plain FP32 path")
    p.add_argument("--stream-full", action="store_true",
                   help="only the scene stream at its stated size: 10,000 queries saturated, Poisson arrivals at "
                        "0.8 of the saturated rate over all of them and at 0.25 / 0.5 over the first 2,000")
    p.add_argument("--serve-burst", type=int, default=200, help="256-object scene queries in the warm burst")
    p.add_argument("--objects", type=int, default=256,
                   help="object count of the matrix workload (256 = the benchmark; smaller only for profiling)")
    p.add_argument("--profile-case", default=None,
                   choices=["contract", "adjoint", "surfel_forward", "surfel_adjoint", "jacobian", "serve"],
                   help="run one kernel family's workload a few times (for ncu captures) instead of the benchmark")
    return p.parse_args()


def dist_setup(n):
    rank, world, local = int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.path or not os.path.exists(self.path):
            return out
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if sm:
            out.update(sm_mhz=statistics.median(sm), sm_max_mhz=max(mx), reasons=sorted(reasons), samples=len(sm))
        return out


def workload_config(meta, n_k, world):
    """The `config` object of both legs (same keys and values for the same workload)."""
    return {"workload": meta["workload"], "n_k": n_k, "n_objects": meta["n_objects"],
            "n_triangles": meta["n_triangles"], "mix": meta["mix"], "seed": "rank (0 at N=1)",
            "l2": "GPU leg: flushed (256 MB write) before every timed step", "parallelism": f"replicas x{world}"}


def cpu_baseline_matrix256(oobjs, kgrid, seconds: float, sample_offset: int = 0):
    """FP64 oracle (the reference algorithm restated; OpenMP over all host
    threads) on a strided subset of k-nodes of the same workload.  oobjs are
    oracle objects, kgrid the (dirs, kmag, w) arrays."""
    from oracle import oracle as orc
    dirs, kmag, w = kgrid
    n_tri = sum(len(o.elems) for o in oobjs)
    Q = len(kmag)
    # calibrate on a tiny sample, then size the stride for ~`seconds`
    stride = 4096
    t0 = time.perf_counter()
    orc.form_factor_matrix(oobjs, dirs, kmag, stride=stride)
    dt = max(time.perf_counter() - t0, 1e-3)
    per_node = dt / len(range(0, Q, stride))
    n_nodes = max(1, int(seconds / per_node))
    stride = max(1, Q // n_nodes)
    sel = np.arange(sample_offset % stride, Q, stride)
    t0 = time.perf_counter()
    J = orc.form_factor_matrix(oobjs, dirs[sel], kmag[sel])
    orc.contract(J, w[sel])
    dt = time.perf_counter() - t0
    evals = n_tri * len(sel)
    return {"value": evals / dt, "unit": UNIT, "cores": orc.max_threads(), "kind": "port",
            "sample": f"{len(sel)} of {Q} k-nodes (every {stride}th) x {n_tri} triangles, form factors + contraction, FP64",
            "seconds": dt, "evals": evals}


def run_reference(args):
    """The reference's CPU algorithm (FP64 oracle port: the reference's own
    CPU path needs Eigen, TBB and libigl) on the host cores.  Inputs come from
    oracle.workloads, byte-identical to the GPU leg's, so nothing of the
    product package is imported or loaded here."""
    rank, world, local = dist_setup(args.gpus)
    if rank != 0:
        return
    from oracle import oracle as orc, workloads
    kg, oobjs, meta = workloads.matrix256(seed=0)
    Q = len(kg[1])
    per_step = max(2.0, min(10.0, 150.0 / max(1, args.steps + args.warmup)))
    for w in range(args.warmup):
        cpu_baseline_matrix256(oobjs, kg, per_step / 4, sample_offset=w)
    secs, evals = [], []
    for s in range(args.steps):
        r = cpu_baseline_matrix256(oobjs, kg, per_step, sample_offset=s + 1)
        secs.append(r["seconds"])
        evals.append(r["evals"])
    v = float(sum(evals) / sum(secs))
    evals_step = meta["n_triangles"] * Q
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(secs) / len(secs), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": workload_config(meta, Q, world),
            "step": ("one bounded sample of the workload: the form factors and contraction of every object at a "
                     "strided subset of the k-nodes (ms_per_step is the measured time of that sample)"),
            "ms_per_full_matrix_extrapolated": 1e3 * evals_step / v,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": orc.max_threads(), "kind": "port",
                             "sample": r["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_gb300(args):
    import torch
    rank, world, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from pointint_gb300 import configs, core, _lib
    peaks, peak_src = load_peaks()
    kg, objs, meta = configs.matrix256(seed=rank, n_objects=args.objects)
    n_obj = len(objs)
    n_tri = meta["n_triangles"]
    Q = kg.num_nodes
    evals_step = n_tri * Q
    # the kernel evaluates one direction of each antipodal pair and writes the
    # other from it (A(-k) = -conj A(k)): its own evaluations, for the roofline
    n_dirs, n_eval_dirs = kg.info()[1], len(kg.direction_pairs())
    evals_kernel = evals_step * n_eval_dirs // n_dirs
    precision = "fp16x3" if args.precision == "auto" else args.precision
    stream = torch.cuda.current_stream()
    batch = core.ObjectBatch(objs)
    Jw = torch.empty((n_obj, Q), dtype=torch.complex64, device="cuda")
    amax = torch.empty(n_obj, dtype=torch.float32, device="cuda")  # row maxima: the FP16 operand scales
    V = torch.empty((n_obj, n_obj), dtype=torch.float64, device="cuda")
    ws = core.Workspace()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    def step(ev_ff=None):
        batch.prepare()
        if ev_ff:
            ev_ff[0].record(stream)
        core.form_factors(kg, batch, True, out=Jw, row_amax=amax)
        if ev_ff:
            ev_ff[1].record(stream)
        core.contract(kg, Jw, precision, out=V, workspace=ws, row_amax=amax)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = _lib.launch_count()
    total_ms, ff_ms = 0.0, 0.0
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step((f0, f1))
            e1.record(stream)
            e1.synchronize()
            total_ms += e0.elapsed_time(e1)
            ff_ms += f0.elapsed_time(f1)
        torch.cuda.synchronize()
    launches = _lib.launch_count() - launches0
    clocks = clk.summary()
    t = torch.tensor([total_ms], dtype=torch.float64, device="cuda")
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.barrier()
    total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = world * evals_step * args.steps / (total_ms / 1e3)

    # contraction alone: FP32 vs the split forms (warm: resident J).  Calls run
    # back to back, `inner` per timed group, so the host's launch work overlaps
    # the previous call's kernels; J (157.5 MB) is larger than L2, and L2 is
    # flushed before each group.
    def time_contract(p, reps=5, inner=10):
        core.contract(kg, Jw, p, out=V, workspace=ws, row_amax=amax)
        torch.cuda.synchronize()
        ms = []
        for _ in range(reps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(inner):
                core.contract(kg, Jw, p, out=V, workspace=ws, row_amax=amax)
            b.record(stream)
            b.synchronize()
            ms.append(a.elapsed_time(b) / inner)
        return statistics.median(ms)

    # FP64 reference of the same contraction (cuBLAS DGEMM: a check, not the product path)
    X = torch.view_as_real(Jw).reshape(n_obj, -1).double()
    V64 = (X @ X.T) / (8 * np.pi ** 3)
    d64 = torch.sqrt(torch.outer(torch.diagonal(V64), torch.diagonal(V64)).abs())

    def cond_err(Vx, eps):
        return ((Vx - V64).abs() / torch.maximum(V64.abs(), eps * d64)).max().item()

    contraction = {"reference": "FP64 contraction of the same J"}
    for p in ("fp32", "tf32x3", "bf16x3", "fp16x3"):
        try:
            contraction[p] = {"ms": time_contract(p), "max_rel_err": cond_err(V, 1e-3),
                              "max_rel_err_floor_1e-2": cond_err(V, 1e-2)}
        except _lib.PointIntError as exc:
            contraction[p] = {"error": str(exc)}
    for p in ("tf32x3", "bf16x3", "fp16x3"):
        if "ms" in contraction.get(p, {}) and "ms" in contraction["fp32"]:
            contraction[f"speedup_{p}_vs_fp32"] = contraction["fp32"]["ms"] / contraction[p]["ms"]
    contraction["error_definition"] = "max_ij |dV_ij| / max(|V_ij|, eps sqrt(V_ii V_jj)), eps = 1e-3 (or 1e-2)"
    contraction["timing"] = ("median over 5 groups of 10 back-to-back calls through pi_contract_rowmax with the "
                             "row maxima the form-factor kernel wrote (host work overlaps the previous call); J "
                             "(157.5 MB) larger than L2, L2 flushed before each group")
    del X, V64

    sm_clock = clocks.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count
    ff_avg_s = ff_ms / args.steps / 1e3
    clk_max = float(peaks.get("sm_max_mhz", 2070.0))
    fp32_achieved = FP32_FLOPS_PER_EVAL * evals_kernel / ff_avg_s / 1e12
    fp32_peak = n_sm * FP32_FLOPS_PER_SM_PER_CLK * clk_max * 1e6 / 1e12
    sfu_achieved = SFU_OPS_PER_EVAL * evals_kernel / ff_avg_s / 1e9
    sfu_peak = n_sm * SFU_PER_SM_PER_CLK * clk_max * 1e6 / 1e9
    # issue slots: 4 warp instructions per SM per clock; thread instructions per
    # evaluation from the kernel's ncu capture on 32 of the 256 objects
    issue_achieved = FF_THREAD_INSTR_PER_EVAL / 32.0 * evals_kernel / ff_avg_s / 1e9
    issue_peak = n_sm * 4 * clk_max * 1e6 / 1e9
    roofline = {"kernel": "ff_kernel", "bound": "fp32-issue", "achieved": fp32_achieved, "peak": fp32_peak,
                "unit": "TFLOP/s", "frac": fp32_achieved / fp32_peak, "traffic": FF_TRAFFIC_BYTES_PER_LAUNCH,
                "kernel_ms": ff_avg_s * 1e3, "share_of_step": (ff_ms / total_ms) if world == 1 else None,
                "algorithmic_unit": f"{FP32_FLOPS_PER_EVAL} FP32 flops (FMA = 2) per triangle x k evaluation, the "
                                    f"reference algorithm's count, x {evals_kernel:.4e} evaluations the kernel "
                                    f"performs: {n_eval_dirs} of the {n_dirs} directions, one of each antipodal pair "
                                    f"(A(-k) = -conj A(k) gives the other); the workload's {evals_step:.4e} "
                                    "triangle x k pairs are all produced",
                "evaluated_directions": {"evaluated": n_eval_dirs, "of": n_dirs},
                "peak_source": f"nominal FP32: {FP32_FLOPS_PER_SM_PER_CLK} flops/clk/SM x {n_sm} SMs x {clk_max} MHz "
                               "(MEASURED_PEAKS.json holds HBM and bf16 tensor peaks only)",
                "binding": "FP32 issue and FMA pipe: no MUFU (SFU) instructions (sine/cosine are a phasor table "
                           "and polynomials); the short-series loop runs two radii per packed FP32 instruction, which "
                           "holds the FMA pipe two cycles, so the FMA pipe (math-pipe throttle, the second stall) and "
                           "the issue slots bind together",
                "pipes_from_capture": {"fma_pipe_active": FF_FMA_PIPE_ACTIVE, "issue_active": FF_ISSUE_ACTIVE,
                                       "source": "ncu --set full of the same kernel on 32 of the 256 objects"},
                "issue": {"thread_instructions_per_evaluation": FF_THREAD_INSTR_PER_EVAL,
                          "achieved": issue_achieved, "peak": issue_peak, "unit": "G warp-instructions/s",
                          "frac": issue_achieved / issue_peak,
                          "source": "instructions per evaluation from ncu (smsp__inst_executed.sum x 32 / "
                                    "evaluations, 32-object capture); rate from this run's CUDA events"},
                "sfu_count": {"achieved": sfu_achieved, "peak": sfu_peak, "unit": "Gop/s", "frac": sfu_achieved / sfu_peak,
                              "note": f"{SFU_OPS_PER_EVAL} SFU-class operations per evaluation in the reference "
                                      "algorithm (accounting only: this kernel issues none)"}}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded)",
            "config": workload_config(meta, Q, world), "contraction_precision": precision,
            "vol_matrix_per_s": world * args.steps / (total_ms / 1e3),
            "contraction": contraction, "clocks": clocks, "gpu_launches": launches, "roofline": roofline,
            "work_note": (f"value counts the workload's {evals_step:.4e} triangle x k pairs per step, all of them "
                          f"produced in J; the form-factor kernel evaluates {evals_kernel:.4e} of them (one direction "
                          f"of each antipodal pair, {n_eval_dirs} of {n_dirs}) and writes the rest as "
                          "A(-k) = -conj A(k)")}

    if rank == 0 and not args.no_e2e:
        line["e2e"] = e2e_host(kg, objs, precision, args.steps, evals_step, world)
    if rank == 0 and not args.no_serve and args.objects == 256:
        line["serving"] = serving_bench(args, kg, objs, batch, contraction, flush)
    if rank == 0 and not args.no_configs and args.objects == 256:
        line["configs"] = configs_bench(args, flush)
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            from oracle import oracle as orc
            oobjs = [orc.Obj(o.geom.type, o.geom.elems, o.dof_type, o.dofs) for o in objs]
            line["cpu_baseline"] = {k: v for k, v in cpu_baseline_matrix256(oobjs, (kg.dirs, kg.kmag, kg.w),
                                                                            args.cpu_seconds).items()
                                    if k not in ("seconds", "evals")}
        except Exception as exc:  # the oracle must not break the GPU line
            line["cpu_baseline"] = {"value": None, "error": str(exc)}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# DRAM bytes (read + write) of one full-size ff_kernel launch.  Reads: captured
# with ncu on 32 of the 256 objects (82,112 triangles: 5.70 MB with the
# centroid low words) and scaled by the triangle count (656,896 / 82,112),
# since element reads grow with the elements.  Writes: that capture's J
# (19.7 MB) stayed in L2, but the full J (256 x 76,928 complex64 = 157.5 MB)
# exceeds the 129 MB L2 and is counted as written once.
FF_TRAFFIC_BYTES_PER_LAUNCH = 5.70e6 * 656896 / 82112 + 256 * 76928 * 8
# Thread instructions per evaluation the kernel performs (one direction of
# each antipodal pair), from its ncu capture on 32 of the 256 objects
# (smsp__inst_executed.sum 4.481e9 x 32 / 3.158e9 evaluations; packed FP32
# instructions count once).
FF_THREAD_INSTR_PER_EVAL = 45.4
# The same capture's FMA-pipe busy share (sm__pipe_fma_cycles_active, 51.0%
# of active cycles, packed FP32 instructions holding the pipe two cycles) and
# issue-slot share (smsp__issue_active, 59.0%).  The 32-object launch is 1.6
# waves of CTAs and ends on a tail (2.8 warps per scheduler on average), so
# both read lower than in the 256-object launch, whose issue share the line's
# `issue.frac` gives from its own time.
FF_FMA_PIPE_ACTIVE = 0.510
FF_ISSUE_ACTIVE = 0.590


def _pcts(ms):
    a = np.sort(np.asarray(ms))
    return {"p50_ms": float(np.percentile(a, 50)), "p99_ms": float(np.percentile(a, 99)), "n": int(len(a))}


def _timed(fn, flush, reps=3):
    """Median CUDA-event time (ms) of fn() over reps runs after one warm-up, L2 flushed before each."""
    import torch
    fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        ts.append(a.elapsed_time(b))
    return statistics.median(ts)


def configs_bench(args, flush):
    """The other workload configurations, each timed on the GPU (samples where
    the full configuration would take more than a few seconds):
      pair_sweep   cube x icosphere-3 at 64 offsets, L=32 x Lebedev-302; volumes
                   checked against the FP64 oracle on 8 of the 64 pairs
      large_mesh   2 of the 32 star-shaped 200,000-triangle solids, L=128 x
                   Lebedev-5810 (N_k = 743,680)
      surfels64    8 of the 64 objects x 50,000 disks, forward volume matrix and
                   the backward pass to per-disk positions and normals"""
    import torch
    from pointint_gb300 import configs, core
    out = {}
    # pair sweep
    kg1, cube, spheres, offsets, meta1 = configs.pair_sweep()
    b1 = core.ObjectBatch([cube] + spheres)
    Jw = torch.empty((len(spheres) + 1, kg1.num_nodes), dtype=torch.complex64, device="cuda")
    V1 = {}

    def sweep():
        core.form_factors(kg1, b1, True, out=Jw)
        V1["V"] = core.contract(kg1, Jw, "fp32")
    ms = _timed(sweep, flush)
    vols = V1["V"][0, 1:].cpu().numpy()
    evals1 = (cube.geom.num_elements() + spheres[0].geom.num_elements()) * kg1.num_nodes * len(spheres)
    try:
        from oracle import oracle as orc
        orc.build()
        ref = [orc.pair_volume(orc.Obj(cube.geom.type, cube.geom.elems, cube.dof_type, cube.dofs),
                               orc.Obj(s.geom.type, s.geom.elems, s.dof_type, s.dofs),
                               (kg1.dirs, kg1.kmag, kg1.w))["volume"] for s in spheres[:8]]
        err = float(np.max(np.abs(vols[:8] - np.array(ref)) / np.maximum(np.abs(ref), 1e-12)))
    except Exception as exc:  # the oracle must not break the GPU line
        err = f"oracle unavailable: {exc}"
    out["pair_sweep"] = {"workload": meta1["workload"], "ms": ms, "tri_k_evals_per_s": evals1 / (ms / 1e3),
                         "pairs_per_s": len(spheres) / (ms / 1e3), "max_rel_err_vs_oracle_8_pairs": err}
    del b1, Jw
    # large mesh sample
    kg3, objs3, meta3 = configs.large_mesh(n_objects=2)
    b3 = core.ObjectBatch(objs3)
    J3 = torch.empty((len(objs3), kg3.num_nodes), dtype=torch.complex64, device="cuda")
    ms = _timed(lambda: core.form_factors(kg3, b3, True, out=J3), flush, reps=2)
    evals3 = meta3["n_triangles_each"] * len(objs3) * kg3.num_nodes
    out["large_mesh"] = {"workload": meta3["workload"], "sample_objects": len(objs3), "n_k": kg3.num_nodes,
                         "ms": ms, "tri_k_evals_per_s": evals3 / (ms / 1e3),
                         "full_config_seconds_at_this_rate": 32 * meta3["n_triangles_each"] * kg3.num_nodes / (evals3 / (ms / 1e3))}
    core.form_factors(kg3, b3, False, out=J3)
    out["large_mesh"].update(oracle_check(J3, objs3, kg3, 1600))
    del b3, J3
    # surfels sample: forward and backward
    kg4, objs4, meta4 = configs.surfels64(n_objects=8)
    scene = core.Scene(kg4, objs4)
    c0, n0 = scene.surfel_params()
    res = {}

    def fwd():
        res["L"] = scene.volume_matrix_of_surfels(c0, n0).sum()

    def fwd_bwd():
        c = c0.clone().requires_grad_(True)
        n = n0.clone().requires_grad_(True)
        scene.volume_matrix_of_surfels(c, n).sum().backward()
        res["g"] = c.grad
    ms_f = _timed(fwd, flush, reps=2)
    ms_fb = _timed(fwd_bwd, flush, reps=2)
    evals4 = sum(o.geom.num_elements() for o in objs4) * kg4.num_nodes
    out["surfels64"] = {"workload": meta4["workload"], "sample_objects": len(objs4), "forward_ms": ms_f,
                        "forward_disk_k_evals_per_s": evals4 / (ms_f / 1e3), "forward_backward_ms": ms_fb,
                        "backward_over_forward": (ms_fb - ms_f) / ms_f}
    out["surfels64"].update(oracle_check(core.form_factors(kg4, scene.batch, False), objs4, kg4, 1500))
    del scene
    out["hessian256"], out["align"] = hessian_align_bench(flush)
    return out


def oracle_check(J, objs, kg, n_nodes):
    """Form factors of the GPU (J [n, Q], unscaled) against the FP64 oracle at
    n_nodes evenly strided k-nodes (every radius band included), and the
    volumes contracted over those nodes from either J."""
    try:
        from oracle import oracle as orc
        Q = kg.num_nodes
        sel = np.unique(np.linspace(0, Q - 1, n_nodes).astype(np.int64))
        Jg = J[:, torch_index(sel)].cpu().numpy()
        Jo = orc.form_factor_matrix([orc.Obj(o.geom.type, o.geom.elems, o.dof_type, o.dofs) for o in objs],
                                    kg.dirs[sel], kg.kmag[sel]).T
        w = kg.w[sel]
        Vg = ((Jg * w) @ Jg.conj().T).real / (8 * np.pi ** 3)
        Vo = ((Jo * w) @ Jo.conj().T).real / (8 * np.pi ** 3)
        d = np.sqrt(np.abs(np.outer(np.diag(Vo), np.diag(Vo))))
        return {"oracle_sample_nodes": int(len(sel)), "kmax_sampled": float(kg.kmag[sel].max()),
                "J_rel_err_vs_oracle": float(np.linalg.norm(Jg - Jo) / np.linalg.norm(Jo)),
                "max_rel_err_vs_oracle": float((np.abs(Vg - Vo) / np.maximum(np.abs(Vo), 1e-3 * d)).max()),
                "error_definition": "volumes over the sampled nodes: max_ij |dV_ij| / max(|V_ij|, 1e-3 sqrt(V_ii V_jj))"}
    except Exception as exc:  # the oracle must not break the GPU line
        return {"max_rel_err_vs_oracle": f"oracle unavailable: {exc}"}


def torch_index(sel):
    import torch
    return torch.as_tensor(sel, device="cuda")


def hessian_align_bench(flush):
    """Gauss-Newton Hessian of the 256-object matrix (DoF Jacobian of 3,072
    rows + FP32 contraction) and the alignment caller (an icosphere-4
    ellipsoid moving onto a box, N_k = 76,928): one similarity evaluation with gradient and
    Hessian, and a full damped-Newton run from the warm start (host wall-clock,
    results read back each evaluation)."""
    import torch
    from pointint_gb300 import align, configs, core, geometry as G
    kg, objs, meta = configs.matrix256()
    b = core.ObjectBatch(objs)
    Gm = torch.empty((12 * len(objs), kg.num_nodes), dtype=torch.complex64, device="cuda")
    ms_j = _timed(lambda: core.dof_jacobian(kg, b, out=Gm), flush, reps=2)
    H = {}
    ms_h = _timed(lambda: H.__setitem__("H", core.contract(kg, Gm, "fp32")), flush, reps=2)
    ms_h16 = _timed(lambda: H.__setitem__("H16", core.contract(kg, Gm, "fp16x3")), flush, reps=2)
    H32, H16 = H["H"], H["H16"]
    dH = torch.sqrt(torch.outer(torch.diagonal(H32), torch.diagonal(H32)).abs())
    err16 = ((H16 - H32).abs() / torch.maximum(H32.abs(), 1e-3 * dH)).max().item()
    D = Gm.shape[0]
    hess = {"workload": meta["workload"] + "; Gauss-Newton Hessian over all 12 x 256 AffineDoFs",
            "dofs": int(D), "jacobian_ms": ms_j, "contraction_ms": ms_h,
            "jacobian_tri_k_evals_per_s": meta["n_triangles"] * kg.num_nodes / (ms_j / 1e3),
            "contraction_tflops": 4.0 * kg.num_nodes * D ** 2 / (ms_h / 1e3) / 1e12,
            "contraction_fp16x3_ms": ms_h16,
            "contraction_fp16x3_max_rel_err_vs_fp32": err16,
            "contraction_error_definition": "max_ij |dH_ij| / max(|H_ij|, 1e-3 sqrt(H_ii H_jj)), FP16x3 against "
                                            "the FP32 contraction of the same Jacobian rows",
            "contraction_flops_definition": "4 N_k D^2 (full matrix)"}
    del Gm, b, H, H32, H16
    torch.cuda.empty_cache()
    rng = np.random.default_rng(0)
    V, F = G.icosphere(4)
    g2 = G.make_triangle_mesh((V * np.array([1.4, 0.9, 0.6])) @ G.random_rotation(rng).T + 0.3, F)
    Vb, Fb = G.box_mesh([1.6, 1.1, 0.8])
    g1 = G.make_triangle_mesh(Vb @ G.random_rotation(rng).T, Fb)
    with align.Aligner(g1, g2, kg) as a:
        V1 = a.fixed_volume()
        d0 = align.compute_warm_start(g1, g2)
        a.similarity(d0, align.SIM_DICE, V1, align.SIM_ALL)
        ts = []
        for _ in range(5):
            t0 = time.perf_counter()
            a.similarity(d0, align.SIM_DICE, V1, align.SIM_ALL)
            ts.append((time.perf_counter() - t0) * 1e3)
        tf = []
        for _ in range(5):
            t0 = time.perf_counter()
            a.similarity(d0, align.SIM_DICE, V1, align.SIM_FUNC_ONLY)
            tf.append((time.perf_counter() - t0) * 1e3)
        s0 = a.similarity(d0, align.SIM_DICE, V1, align.SIM_FUNC_ONLY).similarity
        t0 = time.perf_counter()
        st = a.optimize(d0, align.SIM_DICE, V1, 1e-6, 20, 0.1)
        run_ms = (time.perf_counter() - t0) * 1e3
    al = {"workload": "alignment, Dice: a moving icosphere-4 ellipsoid (5120 tris, axes 1.4/0.9/0.6) onto a "
                      "fixed rotated box (12 tris), N_k = 76,928, from the moment warm start",
          "similarity_grad_hess_ms": statistics.median(ts), "similarity_value_ms": statistics.median(tf),
          "optimize_ms": run_ms, "newton_iterations": st.iteration + 1, "accepted_steps": st.steps,
          "evaluations": st.evaluations, "similarity_start": s0, "similarity_end": st.similarity,
          "status": st.status}
    return hess, al


def serving_bench(args, kg, objs, batch, contraction, flush):
    """Resident-J serving: (a) the 256-object matrix re-queried under jittered
    translations (warm: form factors resident, translations as phases in the
    FP16-split contraction) against the plain FP32 GPU form; (b) a sample of
    the scene stream (N ~ logU[2,512], 20% rotated objects) at saturation and
    under Poisson arrivals at half that rate, against one-query-at-a-time plain
    FP32 (every form factor re-evaluated, FP32 contraction)."""
    import threading
    import torch
    from pointint_gb300 import configs, core, geometry as G
    from pointint_gb300.serving import Server
    out = {}
    n = len(objs)
    rng = np.random.default_rng(7)
    ids = np.arange(n, dtype=np.int32)

    # plain FP32 GPU form of one matrix: DoF transform + form factors + FP32 contraction
    Jw = torch.empty((n, kg.num_nodes), dtype=torch.complex64, device="cuda")
    V = torch.empty((n, n), dtype=torch.float64, device="cuda")
    ws = core.Workspace()
    stream = torch.cuda.current_stream()
    plain = []
    for i in range(4):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        batch.prepare()
        core.form_factors(kg, batch, True, out=Jw)
        core.contract(kg, Jw, "fp32", out=V, workspace=ws)
        b.record(stream)
        b.synchronize()
        if i:
            plain.append(a.elapsed_time(b))
    plain_ms = statistics.median(plain)
    fp32_contract_ms = contraction.get("fp32", {}).get("ms")

    with Server(kg, objs, precision="fp16x3") as srv:
        t0 = time.perf_counter()
        srv.query(ids, None, np.zeros((n, 3)))          # cold: every row evaluated
        cold_s = time.perf_counter() - t0
        seq = []
        for _ in range(30):                                # unloaded latency
            t = srv.submit(ids, None, rng.normal(0.0, 0.5, size=(n, 3)))
            srv.wait(t)
            a, _, c = srv.times(t)
            seq.append((c - a) / 1e6)
            srv.release(t)
        trs = [rng.normal(0.0, 0.5, size=(n, 3)) for _ in range(args.serve_burst)]
        t0 = time.perf_counter()
        ts = [srv.submit(ids, None, tr) for tr in trs]
        for t in ts:
            srv.wait(t)
        burst_s = time.perf_counter() - t0
        lat = []
        for t in ts:
            a, _, c = srv.times(t)
            lat.append((c - a) / 1e6)
        st = srv.stats()
        # accuracy of the last scene: FP64 contraction of the plain path's J for the same objects
        tr = trs[-1]
        moved = [G.SceneObject(o.geom, o.dof_type, np.concatenate([o.dofs[:3] + tr[k], o.dofs[3:]]))
                 for k, o in enumerate(objs)]
        Jm = core.form_factors(kg, core.ObjectBatch(moved), True)
        X = torch.view_as_real(Jm).reshape(n, -1).double()
        R = ((X @ X.T) / (8 * np.pi ** 3)).cpu().numpy()
        del X, Jm
        d = np.sqrt(np.abs(np.outer(np.diag(R), np.diag(R))))
        err = float((np.abs(ts[-1].V - R) / np.maximum(np.abs(R), 1e-3 * d)).max())
    out["scene_vs_oracle"] = serving_oracle_check(kg, objs[:16] + objs[128:144])
    vps = args.serve_burst / burst_s
    out["matrix256_scenes"] = {
        "what": "256-object scene re-queried with per-object translations N(0,0.5^2): resident J, phases fused "
                "into the FP16-split tensor-core contraction, continuous batching, CUDA graphs",
        "vol_matrix_per_s": vps, "burst_queries": args.serve_burst, "burst_latency": _pcts(lat),
        "unloaded_latency": _pcts(seq), "cold_first_query_ms": cold_s * 1e3,
        "max_rel_err_vs_fp64_contraction": err, "precision": "fp16x3",
        "plain_fp32_vol_matrix_per_s": 1e3 / plain_ms, "plain_fp32_ms": plain_ms,
        "speedup_vs_plain_fp32": vps * plain_ms / 1e3,
        "fp32_contraction_only_vol_matrix_per_s": (1e3 / fp32_contract_ms) if fp32_contract_ms else None,
        "speedup_vs_fp32_contraction_only": (vps * fp32_contract_ms / 1e3) if fp32_contract_ms else None,
        "batches": st["batches"], "graph_launches": st["graph_launches"],
        "tuned_items_per_sm": st["tuned_items_per_sm"], "tuned_k_splits": st["tuned_k_splits"]}

    out["scene_stream"] = stream_bench(kg, args.serve_queries, rates=(0.5,), poisson_queries=args.serve_queries,
                                       plain_prefix=args.serve_plain_prefix)
    return out


def serving_oracle_check(kg, objs, dir_stride=16):
    """A served scene (objects translated by N(0, 0.5^2), FP16-split contraction
    with the phases fused) against the FP64 oracle's volumes over the same
    k-nodes: a server on every radius of the grid at every dir_stride-th
    direction (tensor order kept), which bounds the oracle's cost."""
    from pointint_gb300 import geometry as G
    from pointint_gb300.kgrid import KGrid
    from pointint_gb300.serving import Server
    try:
        from oracle import oracle as orc
        M = 1202
        L = kg.num_nodes // M
        sel = (np.arange(L)[:, None] * M + np.arange(0, M, dir_stride)[None, :]).reshape(-1)
        sub = KGrid(kg.dirs[sel], kg.kmag[sel], kg.w[sel])
        n = len(objs)
        tr = np.random.default_rng(11).normal(0.0, 0.5, size=(n, 3))
        with Server(sub, objs, precision="fp16x3", autotune=False) as srv:
            Vs = srv.query(np.arange(n, dtype=np.int32), None, tr)
        moved = [orc.Obj(o.geom.type, o.geom.elems, o.dof_type, np.concatenate([o.dofs[:3] + tr[k], o.dofs[3:]]))
                 for k, o in enumerate(objs)]
        Vo, _, _ = orc.volume_matrix(moved, (sub.dirs, sub.kmag, sub.w))
        d = np.sqrt(np.abs(np.outer(np.diag(Vo), np.diag(Vo))))
        return {"objects": n, "k_nodes": int(len(sel)), "max_rel_err_vs_oracle":
                float((np.abs(Vs - Vo) / np.maximum(np.abs(Vo), 1e-3 * d)).max()),
                "what": f"{n}-object scene (translations N(0,0.5^2)) served in FP16x3 on all {L} radii x every "
                        f"{dir_stride}th direction, against the FP64 oracle's volumes over the same nodes"}
    except Exception as exc:  # the oracle must not break the GPU line
        return {"max_rel_err_vs_oracle": f"oracle unavailable: {exc}"}


def stream_bench(kg, n_queries, rates=(0.5,), poisson_queries=None, plain_prefix=100, seed=2):
    """The scene stream (N ~ logU[2,512] library objects per query, translations
    N(0,0.5^2), rotations with probability 0.2): n_queries submitted at once
    (saturated throughput and latency), then open-loop Poisson arrivals at each
    fraction of the saturated rate in `rates` over the first poisson_queries
    queries, against one-query-at-a-time plain FP32 (every form factor
    evaluated, FP32 contraction) on the first plain_prefix queries.  Latency is
    host wall-clock from submission to the result written."""
    import threading
    import torch
    from pointint_gb300 import configs, core, geometry as G
    from pointint_gb300.serving import Server
    _, lib, queries, _, meta = configs.serving_stream(seed=seed, n_queries=n_queries, kgrid=False)
    poisson_queries = min(poisson_queries or n_queries, n_queries)
    out = {"workload": meta["workload"], "queries": n_queries, "mean_objects": meta["mean_objects"],
           "precision": "fp16x3"}
    with Server(kg, lib, precision="fp16x3") as srv:
        srv.query(np.arange(len(lib), dtype=np.int32), None, None)  # library rows resident
        st0 = srv.stats()
        t0 = time.perf_counter()
        ts = [srv.submit(*q) for q in queries]
        lat = []
        for t in ts:
            srv.wait(t)
            a, _, c = srv.times(t)
            lat.append((c - a) / 1e6)
            srv.release(t)
        sat_s = time.perf_counter() - t0
        qps = n_queries / sat_s
        st = srv.stats()
        out.update(saturated_queries_per_s=qps, saturated_latency=_pcts(lat),
                   evaluations=st["evaluations"] - st0["evaluations"], batches=st["batches"] - st0["batches"])
        sweep = []
        for frac in rates:
            sub = queries[:poisson_queries]
            gaps = np.random.default_rng(3).exponential(1.0 / (frac * qps), size=len(sub))
            tickets = []

            def feed():
                t_start = time.perf_counter()
                due = np.cumsum(gaps)
                for k, q in enumerate(sub):
                    dt = due[k] - (time.perf_counter() - t_start)
                    if dt > 0:
                        time.sleep(dt)
                    tickets.append(srv.submit(*q))

            th = threading.Thread(target=feed)
            t1 = time.perf_counter()
            th.start()
            th.join()
            lat = []
            for t in tickets:
                srv.wait(t)
                a, _, c = srv.times(t)
                lat.append((c - a) / 1e6)
                srv.release(t)
            span = time.perf_counter() - t1
            sweep.append({"rate_fraction_of_saturated": frac, "offered_queries_per_s": frac * qps,
                          "achieved_queries_per_s": len(sub) / span, "queries": len(sub), "latency": _pcts(lat)})
        out["poisson"] = sweep
    # one query at a time, plain FP32: every form factor evaluated, FP32 contraction
    base = []
    for objects, rot, trans in queries[:plain_prefix]:
        sc = [G.SceneObject(lib[o].geom, lib[o].dof_type, G.affine_dofs(rot[k], trans[k]))
              for k, o in enumerate(objects)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        core.volume_matrix(kg, sc, "fp32")
        torch.cuda.synchronize()
        base.append(time.perf_counter() - t0)
    if base:
        out.update(plain_fp32_one_at_a_time_queries_per_s=len(base) / sum(base), plain_fp32_prefix=len(base),
                   plain_fp32_latency=_pcts([b * 1e3 for b in base]),
                   speedup_vs_plain_fp32_one_at_a_time=qps * sum(base) / len(base))
    return out


def e2e_host(kg, objs, precision, steps, evals_step, world):
    """Same metric through pi_volume_matrix_host: host geometry + host k-grid in,
    host V out, uploads and downloads inside the timed region."""
    from pointint_gb300 import core
    core.volume_matrix_host(kg, objs, precision)  # warm-up
    n = len(objs)
    # element arrays named by several objects (instances of one mesh) are
    # uploaded once by the host entry point
    arrays = {o.geom.elems.ctypes.data: o.geom.elems.nbytes for o in objs}
    h2d = sum(arrays.values()) + sum(o.dofs.nbytes for o in objs) + kg.dirs.nbytes + kg.kmag.nbytes + kg.w.nbytes
    d2h = n * n * 8
    reps = max(3, min(steps, 10))
    t0 = time.perf_counter()
    for _ in range(reps):
        core.volume_matrix_host(kg, objs, precision)
    dt = (time.perf_counter() - t0) / reps
    return {"value": world * evals_step / dt, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": d2h,
            "ms_per_step": dt * 1e3, "entry_point": "pi_volume_matrix_host",
            "distinct_element_arrays": len(arrays)}


def profile_case(name: str, n_objects: int = 256):
    """One kernel family's workload, three times (the first launch warms up),
    with CUDA-event times printed as one JSON line.  For ncu captures of the
    kernels that the benchmark line does not time on their own:
      contract        FP32 / TF32x3 / BF16x3 / FP16x3 contractions of the 256-object J
      adjoint         dV/dtheta of the 256-object matrix (W = 1): adj_tri_kernel + chain
      surfel_forward  volume matrix of 8 objects x 50,000 disks (form factors + contraction)
      surfel_adjoint  the same forward plus per-disk position / normal gradients
      jacobian        DoF Jacobian of the 256-object matrix (3,072 rows)
      serve           the 256-object scene re-queried under translations (20 queries)"""
    import torch
    from pointint_gb300 import configs, core
    out = {"case": name}

    def timed(fn, reps=3):
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return ts

    if name in ("contract", "adjoint", "jacobian", "serve"):
        kg, objs, meta = configs.matrix256(n_objects=n_objects)
        batch = core.ObjectBatch(objs)
        J = core.form_factors(kg, batch, True)
        n = len(objs)
        if name == "contract":
            for p in ("fp32", "tf32x3", "bf16x3", "fp16x3"):
                out[p + "_ms"] = timed(lambda: core.contract(kg, J, p))
        elif name == "adjoint":
            W = np.ones((n, n))
            out["ms"] = timed(lambda: core.dof_gradients(kg, batch, J, W))
        elif name == "jacobian":
            G = torch.empty((12 * n, kg.num_nodes), dtype=torch.complex64, device="cuda")
            out["ms"] = timed(lambda: core.dof_jacobian(kg, batch, out=G))
        else:
            from pointint_gb300.serving import Server
            del J
            rng = np.random.default_rng(0)
            ids = np.arange(n, dtype=np.int32)
            with Server(kg, objs, precision="fp16x3", autotune=False) as srv:
                srv.query(ids, None, np.zeros((n, 3)))
                t0 = time.perf_counter()
                for _ in range(20):
                    srv.query(ids, None, rng.normal(0.0, 0.5, size=(n, 3)))
                out["ms_per_query"] = (time.perf_counter() - t0) * 1e3 / 20
    else:
        kg, objs, meta = configs.surfels64(n_objects=8)
        scene = core.Scene(kg, objs)
        c0, n0 = scene.surfel_params()

        def fwd_bwd():
            c = c0.clone().requires_grad_(True)
            nn = n0.clone().requires_grad_(True)
            scene.volume_matrix_of_surfels(c, nn).sum().backward()
        out["ms"] = timed(fwd_bwd if name == "surfel_adjoint" else lambda: scene.volume_matrix_of_surfels(c0, n0))
    out["workload"] = meta["workload"]
    print(json.dumps(out))


def main():
    args = parse()
    if args.stream_full:
        import torch
        from pointint_gb300.kgrid import standard_kgrid
        torch.cuda.set_device(0)
        line = {"mode": "scene stream, full size", "metric": "queries/s; p50/p99 latency ms",
                "stream": None}
        kg = standard_kgrid(59, 64)
        res = stream_bench(kg, 10000, rates=(0.8,), poisson_queries=10000, plain_prefix=args.serve_plain_prefix)
        low = stream_bench(kg, 2000, rates=(0.25, 0.5), poisson_queries=2000, plain_prefix=0)
        res["poisson"] = low["poisson"] + res["poisson"]
        line["stream"] = res
        print(json.dumps(line))
        return
    if args.profile_case:
        profile_case(args.profile_case, args.objects)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
