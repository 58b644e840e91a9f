#!/usr/bin/env python
"""Benchmark of the GB300 FV3 tracer-transport path.

Metric: tracer-cell-level updates/s, one update = one tracer value of one cell
of one level advanced by a full step = tracer_2d (n_split substeps of
fv_tp_2d + flux-form update) followed by the map_scalar kord=9 remap of every
tracer onto the hybrid levels.  Workload: six C384 tiles, 127 levels,
20 tracers, n_split=3, hord_tr=8, kord=9, seeded synthetic fields (no public
dataset exists for this path): cosine bells / Gaussian blobs with 1 % noise,
solid-body rotation tilted 45 deg plus a degree-20 spherical-harmonic stream
function perturbation (10 m/s), max Courant 0.8, Lagrangian delp perturbed
+-10 % per layer with column mass kept, ps in 950-1030 hPa.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Legs (rank 0 prints ONE JSON line): the FP32-mixed path (headline, CUDA
graph per step), the FP64 path, the mixed-vs-FP64 error per tracer and the
global mass drift, the end-to-end C-ABI path with pinned host buffers, the
roofline of the advection substep kernel, and the CPU oracle baseline.
With N > 1 ranks each GPU advances an independent ensemble member (replicas,
weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "tracer-cell-level updates/s at C384L127: FP32-mix vs FP64 on 1 GB300; % HBM"
UNIT = "tracer-cell-level updates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="fv3g", choices=["fv3g", "reference"])
    ap.add_argument("--resolution", dest="n", type=int, default=384, help="cells per tile edge (C_n)")
    ap.add_argument("--npz", type=int, default=127)
    ap.add_argument("--nq", type=int, default=20)
    ap.add_argument("--q-split", type=int, default=3)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--groups", type=int, default=0,
                    help="tracer groups of the pipelined e2e step (0 = nq / warps per CTA)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--warps", type=int, default=0,
                    help="advection warps per CTA (0 = chosen by fv3g_state_autotune)")
    ap.add_argument("--restart", action="store_true",
                    help="instead of the step: time writing and reading one tile's fv_tracer.res file")
    ap.add_argument("--restart-tracers", type=int, default=4)
    ap.add_argument("--restart-dir", default="", help="where the restart leg writes its file (default: a temp dir)")
    return ap.parse_args()


def workload(a) -> dict:
    return {"workload": f"6xC{a.n} L{a.npz} {a.nq} tracers: tracer_2d n_split={a.q_split} hord_tr=8 + map_scalar kord=9",
            "tiles": 6, "n": a.n, "npz": a.npz, "nq": a.nq, "n_split": a.q_split, "hord": 8, "kord": 9,
            "l2_policy": "inputs larger than L2 (q alone is 9.3 GB FP32 / 18.5 GB FP64 vs 129 MB L2)"}


def alg_bytes(a, s_q: int, s_f: int) -> dict:
    """Algorithmic HBM bytes (halo cells excluded): per substep launch and per step."""
    cells = 6 * a.n * a.n * a.npz
    sub = cells * (a.nq * 2 * s_q + 8 * s_f)      # q in/out + cx,cy,xfx,yfx,mfx,mfy,dp1 in, dp2 out
    rem = cells * (a.nq * 2 * s_q + 2 * s_f)      # q in/out + delp in, delp out
    return {"substep": sub, "remap": rem, "step": a.q_split * sub + rem,
            "per_update": (a.q_split * sub + rem) / (cells * a.nq)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def op_ceiling(q_split: int, updates_per_s: float, sm_max_mhz):
    """Secondary (compute) ceiling: the oracle's counted operations per update (tests/golden/op_counts.json,
    written by tests/golden/make_golden.py) times the update rate, against the nominal FP32 (non-tensor)
    rate of the GPU's SMs at their maximum clock."""
    try:
        with open(os.path.join(ROOT, "tests", "golden", "op_counts.json")) as f:
            c = json.load(f)
    except (OSError, ValueError):
        return None
    flops = q_split * c["flops_per_substep_cell"] + c["flops_per_remap_level"]
    ops = q_split * c["ops_per_substep_cell"] + c["ops_per_remap_level"]
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count if torch.cuda.is_available() else 152
    mhz = float(sm_max_mhz) if sm_max_mhz else 2070.0
    peak = sms * 128 * 2 * mhz * 1e6 / 1e12  # 128 FP32 lanes per SM, an FMA counted as two flops
    achieved = updates_per_s * flops / 1e12
    return {"flops_per_update": flops, "ops_per_update": ops, "achieved_tflops": achieved,
            "achieved_tops": updates_per_s * ops / 1e12, "peak_tflops_fp32_nominal": peak,
            "frac": achieved / peak,
            "source": "oracle op-counting scalar: +,-,*,/ on tracer values (ops adds min/max/sign)",
            "peak_kind": f"nominal: {sms} SMs x 128 FP32 lanes x 2 x {mhz:.0f} MHz"}


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def committed_traffic(precision: str):
    """DRAM bytes of one substep (interior + edge-ring launches) at this workload from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "substep_kernel_C384L127x20.txt")
    try:
        with open(path) as f:
            txt = f.read()
    except OSError:
        return None
    m = re.search(rf"traffic_per_substep_{precision}_bytes\s*[:=]\s*([0-9.eE+]+)", txt)
    return float(m.group(1)) if m else None


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        # the raw samples; FV3G_CLOCKS_DIR picks where they are kept (default: the temp directory)
        import tempfile
        self.path = os.path.join(os.environ.get("FV3G_CLOCKS_DIR", tempfile.gettempdir()), f"clocks_rank{index}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 8:
                    rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[4 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((float(r[2]) for r in rows if re.match(r"^[0-9.]+$", r[2])), default=None)}


# ----------------------------------------------------------------- helpers --
def dist_setup():
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# Ensemble configuration: 32 single-tile members (16 x C48 L32, 10 x C96 L64,
# 6 x C192 L127), 4 tracers each, Courant <= 0.7, n_split 2, hord 8, kord 9.
ENSEMBLE = [(48, 32)] * 16 + [(96, 64)] * 10 + [(192, 127)] * 6


def ensemble_leg(a, stream):
    """The uneven ensemble (16 x C48 L32, 10 x C96 L64, 6 x C192 L127 single tiles, 4 tracers each), mixed
    precision.  Headline form: the members of each size as one state of independent tiles (one launch per
    phase for all of them), the three states on three streams of one CUDA graph per step
    (fv3g_ensemble_step), each state's CTA width autotuned; per-member error of one step against the FP64
    path (each member against the oracle: tests/test_gpu_configs.py).  Also timed: one state per member in
    the same graph form (per_member_states)."""
    import numpy as np
    import torch
    from fv3atm_gb300 import api
    from fv3atm_gb300 import synth as S
    probs = [S.make_problem(n, npz, 4, ntiles=1, seed=5000 + k, cmax=0.7) for k, (n, npz) in enumerate(ENSEMBLE)]
    units = sum(n * n * npz * 4 for n, npz in ENSEMBLE)
    s = stream.cuda_stream

    def timed(ens):
        for _ in range(max(1, min(a.warmup, 3))):
            ens.step(2, stream=s)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(a.steps):
            ens.step(2, stream=s)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / a.steps

    # one state of independent tiles per size
    sizes = sorted(set(ENSEMBLE))
    batches, widths = [], {}
    for n, npz in sizes:
        B = S.stack_tiles([P for P, sz in zip(probs, ENSEMBLE) if sz == (n, npz)])
        st = api.CubeState(n, npz, 4, precision="mixed", ntiles=B.ntiles, independent_tiles=True)
        st.load_problem(B)
        widths[f"C{n}L{npz}x{B.ntiles}"] = st.autotune()
        batches.append((st, B))
    ens = api.Ensemble([st for st, _ in batches])
    ens.step(2, stream=s)  # accuracy: one step from the initial fields against the FP64 path
    torch.cuda.synchronize()
    errs = []
    for st, B in batches:
        ref = api.CubeState(B.n, B.npz, 4, precision="fp64", ntiles=B.ntiles, independent_tiles=True)
        ref.load_problem(B)
        ref.step(2)
        g, r = st.download("Q_REMAPPED"), ref.download("Q_REMAPPED")
        for t in range(B.ntiles):
            sl = (t, slice(None), slice(None), slice(3, 3 + B.n), slice(3, 3 + B.n))
            errs.append(float(np.linalg.norm((g - r)[sl]) / np.linalg.norm(r[sl])))
        ref.close()
    for st, B in batches:  # back to the initial fields
        st.upload("Q", B.q.numpy())
    ms = timed(ens)
    ens.close()
    for st, _ in batches:
        st.close()
    # one state per member, the same graph form
    states = []
    for P in probs:
        st = api.CubeState(P.n, P.npz, 4, precision="mixed", ntiles=1)
        st.load_problem(P)
        st.autotune()
        states.append(st)
    ens = api.Ensemble(states)
    ms_members = timed(ens)
    ens.close()
    for st in states:
        st.close()
    return {"value": units / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "members": len(ENSEMBLE),
            "rel_l2_vs_fp64_max": max(errs), "rel_l2_vs_fp64_mean": sum(errs) / len(errs),
            "warps_per_cta_by_size": widths,
            "per_member_states": {"value": units / (ms_members / 1e3), "ms_per_step": ms_members},
            "config": "16 x C48 L32 + 10 x C96 L64 + 6 x C192 L127 single tiles (prescribed halo ring), 4 tracers, "
                      "n_split 2, hord 8, kord 9, mixed precision; the members of each size as one state of "
                      "independent tiles, one graph per ensemble step"}


def build_state(P, precision, nq, npz, n, warps=0):
    import torch
    from fv3atm_gb300 import api
    st = api.CubeState(n, npz, nq, precision=precision, hord=8, kord=9, warps_per_cta=warps)
    st.set_grid(P.geoms)
    st.set_levels(P.ak, P.bk)
    dt = torch.float64 if precision == "fp64" else torch.float32
    cur = torch.cuda.current_stream().cuda_stream  # copies are ordered after the conversions
    for name, val in (("Q", P.q), ("DELP", P.dp), ("CX", P.cx), ("CY", P.cy), ("MFX", P.mfx), ("MFY", P.mfy)):
        v = val.to(dt).contiguous()
        st.upload_device(name, v.data_ptr(), stream=cur)
        torch.cuda.synchronize()
        del v
    return st


def timed_steps(st, a, world, steps, warmup, stream):
    """Warm-up, then `steps` graph replays bracketed by barrier + synchronize; per-kernel event times."""
    import torch
    st.set_timing(True)
    for _ in range(warmup):
        st.step(a.q_split, use_graph=True, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    kern = {}
    with torch.cuda.stream(stream):
        e0.record(stream)
        for _ in range(steps):
            st.step(a.q_split, use_graph=True, stream=stream.cuda_stream)
            for k, (ms, cnt) in st.kernel_times().items():
                kms, kc = kern.get(k, (0.0, 0))
                kern[k] = (kms + ms, kc + cnt)
        e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    return max_over_ranks(ms, world), kern


def rel_err_per_tracer(x, ref, n):
    import torch
    s = slice(3, 3 + n)
    out = []
    for iq in range(x.shape[1]):
        a = x[:, iq, :, s, s].double()
        b = ref[:, iq, :, s, s].double()
        out.append(float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b)))
    return out


# ------------------------------------------------------------- CPU oracle --
# The CPU sample of both the reference arm and the cpu_baseline leg: the
# workload's six tiles and levels with CPU_SAMPLE_NQ of its tracers (the
# oracle parallelises over (tile, level), so keeping all levels keeps its
# thread load that of the full workload; per update the cost does not depend
# on the tracer count beyond the per-level setup shared by the tracers).
CPU_SAMPLE_NQ = 2
CPU_SAMPLE_STEPS = 2


def headline_problem(a, rank: int = 0, nq: int = 0):
    """The seeded synthetic problem of the workload (six C{n} tiles, npz levels, nq tracers -- the workload's
    when 0), generated on the GPU when there is one.  Tracers are drawn one by one, so the first tracers of a
    smaller problem equal those of the workload's."""
    import torch
    from fv3atm_gb300 import synth as S
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    return S.make_problem(a.n, a.npz, nq or a.nq, seed=2000 + rank, cmax=0.8, pert_amp=10.0, dp_noise=0.10,
                          device=dev)


def oracle_sample(P, ntr: int) -> dict:
    """Host FP64 copies of the fields of the CPU sample: tracers 0..ntr-1 of P and every per-level field."""
    import numpy as np
    host = lambda t: np.ascontiguousarray(t.detach().to("cpu", dtype=__import__("torch").float64).numpy())  # noqa: E731
    return {"q": host(P.q[:, :ntr]), "dp": host(P.dp), "mfx": host(P.mfx), "mfy": host(P.mfy), "cx": host(P.cx),
            "cy": host(P.cy), "geoms": P.geoms, "topo": P.topo, "ak": P.ak, "bk": P.bk, "n": P.n, "npz": P.npz,
            "nq": ntr}


def cpu_oracle_rate(smp: dict, q_split: int, steps: int, warmup: int = 0):
    """Updates/s of the FP64 C++ oracle (OpenMP, all host threads) on the sample, one step = tracer_2d (q_split
    substeps) + the kord-9 remap of every sample tracer; also returns the remapped tracers of the last step
    (ntr, npz, 6, n, n)."""
    import numpy as np
    import oracle as O
    n, npz, nq = smp["n"], smp["npz"], smp["nq"]
    q0, dp, mfx, mfy, cx, cy = (smp[k] for k in ("q", "dp", "mfx", "mfy", "cx", "cy"))
    sl = slice(3, 3 + n)

    def one_step():
        q1, dp_last, ns = O.tracer_2d_cube(q0, dp, mfx, mfy, cx, cy, smp["geoms"], smp["topo"], hord=8,
                                           q_split=q_split)
        fr = 1.0 / ns
        dpf = dp_last.copy()
        for t, g in enumerate(smp["geoms"]):
            mx, my = mfx[t] * fr, mfy[t] * fr
            dpf[t][:, sl, sl] = dp_last[t][:, sl, sl] + (mx[..., :-1] - mx[..., 1:] + my[..., :-1, :] -
                                                         my[..., 1:, :]) * g.rarea[sl, sl]
        dpi = dpf[:, :, sl, sl].transpose(1, 0, 2, 3).reshape(npz, -1)
        pe1 = np.concatenate([np.full((1, dpi.shape[1]), smp["ak"][0]), smp["ak"][0] + np.cumsum(dpi, axis=0)])
        pe2 = smp["ak"][:, None] + smp["bk"][:, None] * pe1[-1][None]
        return np.stack([O.remap_columns(pe1, q1[:, iq][:, :, sl, sl].transpose(1, 0, 2, 3).reshape(npz, -1), pe2,
                                         kord=9).reshape(npz, 6, n, n) for iq in range(nq)])

    for _ in range(warmup):
        one_step()
    t0 = time.perf_counter()
    for _ in range(steps):
        out = one_step()
    el = time.perf_counter() - t0
    upd = 6 * n * n * npz * nq * steps
    return upd / el, out, {"sample": f"6xC{n} L{npz}, tracers 0..{nq - 1} of the workload's seeded fields, "
                                     f"n_split={q_split}, {steps} steps", "seconds": el, "threads": os.cpu_count()}


def rel_l2_vs_oracle(x, ref, n):
    """Per-tracer relative L2 of a GPU result x (6, ntr, npz, nd, nd) against the oracle's (ntr, npz, 6, n, n)."""
    import numpy as np
    s = slice(3, 3 + n)
    out = []
    for iq in range(ref.shape[0]):
        g = np.asarray(x[:, iq, :, s, s], dtype=np.float64).transpose(1, 0, 2, 3)
        out.append(float(np.linalg.norm(g - ref[iq]) / np.linalg.norm(ref[iq])))
    return out


# ------------------------------------------------------------------- main --
def run_reference(a, world, rank):
    if rank != 0:
        return
    import oracle
    oracle.build()
    P = headline_problem(a, nq=CPU_SAMPLE_NQ)
    smp = oracle_sample(P, CPU_SAMPLE_NQ)
    del P
    rate, _, info = cpu_oracle_rate(smp, a.q_split, steps=a.steps, warmup=a.warmup)
    cfg = workload(a)
    cores = os.cpu_count()
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": 1e3 * info["seconds"] / max(a.steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": cfg,
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "cpu_model": cpu_model(),
                             "sample": info["sample"] + " (C++ FP64 oracle, OpenMP; the upstream Fortran is absent)"},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def restart_leg(a) -> None:
    """Write and read back tile 1's fv_tracer.res file of a mixed state (C{n} L{npz}, restart_tracers tracers)
    through the library, FP64 and FP32 files; the best of three wall times of each call, over the file's bytes.
    The read follows the write, so its file is served from the page cache."""
    import shutil
    import tempfile

    import torch

    import __graft_entry__
    __graft_entry__.build()
    from fv3atm_gb300 import restart as R
    from fv3atm_gb300 import synth as S
    nq = a.restart_tracers
    P = S.make_problem(a.n, a.npz, nq, seed=2000, cmax=0.8, device="cuda")
    st = build_state(P, "mixed", nq, a.npz, a.n)
    names = [f"tracer{i + 1}" for i in range(nq)]
    d = tempfile.mkdtemp(prefix="fv3g_restart_", dir=a.restart_dir or None)
    path = os.path.join(d, "fv_tracer.res.tile1.nc")
    legs = {}
    try:
        for dtype in ("double", "float"):
            tw, tr = [], []
            for _ in range(3):
                t0 = time.perf_counter()
                sums_w = R.write_state(st, "Q", 0, path, names, dtype=dtype)
                tw.append(time.perf_counter() - t0)
                t0 = time.perf_counter()
                sums_r = R.read_state(st, "Q", 0, path, names)
                tr.append(time.perf_counter() - t0)
                assert sums_r == sums_w
            size = os.path.getsize(path)
            legs[dtype] = {"file_bytes": size, "write_GBps": round(size / min(tw) / 1e9, 2),
                           "read_GBps": round(size / min(tr) / 1e9, 2), "write_s": round(min(tw), 4),
                           "read_s": round(min(tr), 4)}
    finally:
        shutil.rmtree(d, ignore_errors=True)
    torch.cuda.synchronize()
    print(json.dumps({"metric": "fv_tracer.res write and read throughput, one tile", "unit": "GB/s of file",
                      "config": {"workload": f"tile 1 of C{a.n} L{a.npz}, {nq} tracers, FP32-mixed state, CDF-2"},
                      "legs": legs, "device": torch.cuda.get_device_name(0)}))


def main():
    a = parse()
    world, rank, local = dist_setup()
    if a.impl == "reference":
        run_reference(a, world, rank)
        return
    if a.restart:
        if rank == 0:
            restart_leg(a)
        return
    import numpy as np
    import torch

    import __graft_entry__
    __graft_entry__.build()

    units = 6 * a.n * a.n * a.npz * a.nq  # tracer-cell-levels per step
    # Pinned host arrays of the end-to-end leg, allocated first, as a model
    # allocates its state at start-up: on this host, pinned blocks taken after
    # the process has churned through tens of GB read back at a fraction of the
    # link bandwidth.
    nd = a.n + 6
    e2e_shapes = {"Q": (6, a.nq, a.npz, nd, nd), "DELP": (6, a.npz, nd, nd), "CX": (6, a.npz, nd, a.n + 1),
                  "CY": (6, a.npz, a.n + 1, nd), "MFX": (6, a.npz, a.n, a.n + 1), "MFY": (6, a.npz, a.n + 1, a.n),
                  "Q_REMAPPED": (6, a.nq, a.npz, nd, nd)}
    pinned = {} if a.no_e2e else {k: torch.empty(v, dtype=torch.float32, pin_memory=True)
                                  for k, v in e2e_shapes.items()}
    t_gen = time.perf_counter()
    P = headline_problem(a, rank)
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t_gen
    stream = torch.cuda.Stream()
    peak, peak_kind = measured_peak()
    out = {}

    # --------------------------------------------------- mixed headline leg
    st = build_state(P, "mixed", a.nq, a.npz, a.n, a.warps)
    warps = a.warps if a.warps > 0 else st.autotune()
    ring_warps = st.widths()[1]
    pairs = st.tracer_pairs()
    m0 = st.mass("Q")
    st.step(a.q_split, use_graph=False)
    st.sync()
    m1 = st.mass("Q_REMAPPED")
    # one step from the initial fields, kept for the comparisons with the FP64 leg and the oracle
    mq = torch.empty(st.field_shape("Q_REMAPPED"), dtype=torch.float32, device="cuda")
    st.download_device("Q_REMAPPED", mq.data_ptr(), stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    mq_sample = mq[:, :CPU_SAMPLE_NQ].cpu().numpy()
    if a.no_fp64:
        del mq
    q32 = P.q.to(torch.float32).contiguous()
    st.upload_device("Q", q32.data_ptr(), stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    del q32
    with ClockSampler(local) as clk:
        ms, kern = timed_steps(st, a, world, a.steps, a.warmup, stream)
    clocks = clk.summary()
    device_error = st.error_code()  # sticky word of the steps: 0 = inputs finite, Courant <= 1, dp > 0
    value = world * units * a.steps / (ms / 1e3)
    ab = alg_bytes(a, 4, 4)
    # one substep = the interior launch + the edge-ring launch of k_substep
    sub_ms, sub_n = kern.get("substep", (0.0, 0))
    sub_avg = sub_ms / (a.steps * a.q_split)
    achieved = ab["substep"] / (sub_avg / 1e3) / 1e9 if sub_avg > 0 else None
    step_gbs = ab["step"] * a.steps / (ms / 1e3) / 1e9
    launches = sum(v[1] for v in kern.values())

    # ------------------------------------------------------ mass-fixer leg
    # the same state with the global mass fixer on: one step's mass change
    # from the initial fields, then the cost of the fixer in timed steps
    st.set_mass_fix(True)
    q32 = P.q.to(torch.float32).contiguous()
    st.upload_device("Q", q32.data_ptr(), stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    del q32
    fm0 = st.mass("Q")
    st.step(a.q_split, use_graph=False)
    st.sync()
    fm1 = st.mass("Q_REMAPPED")
    ms_fix, kern_fix = timed_steps(st, a, world, a.steps, min(a.warmup, 3), stream)
    st.set_mass_fix(False)
    mass_fix = {"rel_change_one_step": [float(abs(x - y) / abs(y)) for x, y in zip(fm1, fm0)],
                "ms_per_step": ms_fix / a.steps, "overhead_ms_per_step": (ms_fix - ms) / a.steps,
                "remap_ms_per_step": kern_fix.get("remap", (0.0, 0))[0] / a.steps,
                "kernels": "per remap: k_mass_partial + reduce before (step-start mass) and after, k_mass_fix"}

    # --------------------------------------------------------------- e2e leg
    e2e = None
    if not a.no_e2e:
        fields_in = ["Q", "DELP", "CX", "CY", "MFX", "MFY"]
        host = {}
        src = {"Q": P.q, "DELP": P.dp, "CX": P.cx, "CY": P.cy, "MFX": P.mfx, "MFY": P.mfy}
        for name in fields_in:
            h = pinned[name]
            assert tuple(h.shape) == tuple(st.field_shape(name)), name
            h.copy_(src[name].to(torch.float32).cpu())
            host[name] = h
        hout = pinned["Q_REMAPPED"]
        assert tuple(hout.shape) == tuple(st.field_shape("Q_REMAPPED"))
        h2d = sum(h.numel() * 4 for h in host.values())
        d2h = hout.numel() * 4
        s = stream.cuda_stream

        marks = []

        def e2e_step():
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            ev[0].record(stream)
            for name in fields_in:
                st.upload_async(name, host[name].data_ptr(), True, s)
            ev[1].record(stream)
            st.step(a.q_split, use_graph=True, stream=s)
            ev[2].record(stream)
            st.download_async("Q_REMAPPED", hout.data_ptr(), True, s)
            ev[3].record(stream)
            marks.append(ev)

        fptr = {k: h.data_ptr() for k, h in host.items()}

        def e2e_pipelined():
            st.step_host(a.q_split, host["Q"].data_ptr(), fptr, hout.data_ptr(), True, a.groups, stream=s)

        st.set_timing(False)
        for _ in range(max(1, min(a.warmup, 2))):
            e2e_step()
            e2e_pipelined()
        torch.cuda.synchronize()
        # link check in this process: one plain pinned copy of the largest input
        probe = torch.empty(host["Q"].numel(), dtype=torch.float32, device="cuda")
        l0, l1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0.record(stream)
        with torch.cuda.stream(stream):
            probe.copy_(host["Q"].view(-1), non_blocking=True)
        l1.record(stream)
        torch.cuda.synchronize()
        link_h2d = host["Q"].numel() * 4 / (l0.elapsed_time(l1) / 1e3) / 1e9
        del probe
        torch.cuda.synchronize()
        barrier(world)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(a.steps):
                e2e_step()
            e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        ems_seq = max_over_ranks(e0.elapsed_time(e1), world)
        timed = marks[-a.steps:]
        phase = {k: sum(ev[i].elapsed_time(ev[i + 1]) for ev in timed) / a.steps
                 for i, k in enumerate(("h2d_ms", "step_ms", "d2h_ms"))}
        # the headline e2e: the pipelined host-array step (transfers of tracer groups overlap the compute)
        torch.cuda.synchronize()
        barrier(world)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(a.steps):
                e2e_pipelined()
            e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        ems = max_over_ranks(e0.elapsed_time(e1), world)
        e2e = {"value": world * units * a.steps / (ems / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": ems / a.steps,
               "host_dtype": "f32 (as a 32BIT build of the model holds its tracers)",
               "path": "fv3g_step_host (the first tracer group in level blocks: upload block b+1 | advect block b; "
                       "later groups: upload g+1 | advect + remap g | download g-1; remap tile by tile with "
                       "each tile's download)",
               # the library's default: one group when the first group streams in level blocks (cube, fixed
               # q_split, at least 16 levels), else groups of one CTA width of tracers
               "groups": a.groups if a.groups > 0 else (1 if a.q_split > 0 and a.npz >= 16 else max(1, a.nq // warps)),
               "sequential": {"value": world * units * a.steps / (ems_seq / 1e3), "ms_per_step": ems_seq / a.steps,
                              "phases": phase, "link_h2d_gbs_plain_copy": link_h2d,
                              "path": "fv3g_upload_async x6 -> fv3g_step (graph) -> fv3g_download_async"}}
        del host, hout
    st.close()

    # ------------------------------------------------------- ensemble leg
    ens = None
    if not a.no_ensemble and world == 1:
        ens = ensemble_leg(a, stream)

    # ---------------------------------------------------- FP64 reference leg
    # Runs after the FP32 legs: its ~80 GB of device allocations and frees
    # leave host-to-device copies from pinned memory several times slower for
    # the rest of the process on this host, which would distort the e2e leg.
    err = None
    fp64_sample = None
    if not a.no_fp64:
        st = build_state(P, "fp64", a.nq, a.npz, a.n, 0)
        st.step(a.q_split, use_graph=False)
        st.sync()  # the step ran on the state's stream; the copy below runs on torch's
        ref_q = torch.empty(st.field_shape("Q_REMAPPED"), dtype=torch.float64, device="cuda")
        st.download_device("Q_REMAPPED", ref_q.data_ptr(), stream=torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        err = rel_err_per_tracer(mq, ref_q, a.n)
        fp64_sample = ref_q[:, :CPU_SAMPLE_NQ].cpu().numpy()
        del mq, ref_q
        torch.cuda.empty_cache()
        ms64, kern64 = timed_steps(st, a, world, max(1, a.steps), max(1, min(a.warmup, 3)), stream)
        out["fp64"] = {"value": world * units * a.steps / (ms64 / 1e3), "ms_per_step": ms64 / a.steps,
                       "kernel_ms_per_step": {k: v[0] / a.steps for k, v in kern64.items()}}
        st.close()
        del st
        torch.cuda.empty_cache()

    # ---------------------------------------------------------- CPU oracle
    cpu = None
    vs_oracle = None
    if rank == 0 and world == 1 and not a.no_cpu:
        smp = oracle_sample(P, CPU_SAMPLE_NQ)
        rate, ref, info = cpu_oracle_rate(smp, a.q_split, steps=CPU_SAMPLE_STEPS, warmup=0)
        cpu = {"value": rate, "unit": UNIT, "cores": info["threads"], "kind": "port", "cpu_model": cpu_model(),
               "sample": info["sample"] + f", {info['seconds']:.1f} s (C++ FP64 oracle, OpenMP)"}
        # the same tracers after one step of the GPU legs, against the FP64 oracle
        vs_oracle = {"tracers": list(range(CPU_SAMPLE_NQ)),
                     "mixed_rel_l2_vs_oracle_per_tracer": rel_l2_vs_oracle(mq_sample, ref, a.n),
                     "fp64_rel_l2_vs_oracle_per_tracer": (rel_l2_vs_oracle(fp64_sample, ref, a.n)
                                                          if fp64_sample is not None else None)}
        del smp, ref

    if rank != 0:
        return
    # the committed ncu summary covers the default workload only
    default = (a.n, a.npz, a.nq, a.q_split) == (384, 127, 20, 3)
    traffic = committed_traffic("mixed") if default else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 stencils; f64 pe/overlap schedule/mass sums", "data": "synthetic (seeded; no public dataset)",
        "config": {**workload(a), "precision": "mixed", "replicas": world, "warps_per_cta": warps,
                   "warps_per_cta_edge_ring": ring_warps, "tracers_per_warp": 2 if pairs else 1},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "kernel": ("k_substep_pair (two tracers per warp)" if pairs else "k_substep<float,8>") +
                               " (fused fv_tp_2d + flux-form update), interior + edge-ring launch pair of one substep",
                     "alg_bytes_per_substep": ab["substep"], "avg_substep_ms": sub_avg,
                     "launches_per_substep": sub_n / (a.steps * a.q_split), "peak_kind": peak_kind},
        "step_hbm": {"alg_bytes_per_update": ab["per_update"], "achieved_gbs": step_gbs, "frac": step_gbs / peak},
        "step_ops": op_ceiling(a.q_split, value / world, (clocks or {}).get("sm_max_mhz")),
        "kernel_ms_per_step": {k: v[0] / a.steps for k, v in kern.items()},
        "gpu_launches": launches,
        "device_error": device_error,
        "clocks": clocks,
        "fp64": out.get("fp64"),
        "mixed_over_fp64": (value / out["fp64"]["value"]) if "fp64" in out else None,
        "mixed_rel_l2_vs_fp64_per_tracer": err,
        "mixed_rel_l2_vs_oracle_per_tracer": vs_oracle["mixed_rel_l2_vs_oracle_per_tracer"] if vs_oracle else None,
        "fp64_rel_l2_vs_oracle_per_tracer": vs_oracle["fp64_rel_l2_vs_oracle_per_tracer"] if vs_oracle else None,
        "mixed_mass_rel_change_one_step": [float(abs(x - y) / abs(y)) for x, y in zip(m1, m0)],
        "mixed_mass_fix": mass_fix,
        "e2e": e2e,
        "ensemble": ens,
        "cpu_baseline": cpu,
        "setup_s": {"generate": t_gen},
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
