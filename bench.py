"""Benchmark of the batched rigid-body step on GB300.

Workload (default): the precision-form configuration, 16384 worlds x 32 bodies
(16 spheres + 16 cubes; radius / half-extents U[0.25,1]; positions
U([-6,6]x[0.5,25]x[-6,6]); velocities U[-2,2]^3; angular velocities
U[-1,1]^3), ground plane y = 0, dt = 1/60, ResolveContacts(4 * len(contacts)).
Synthetic seeded scenes (there is no dataset).

One benchmark "step" is one 600-frame rollout of all worlds from the same
initial state, captured as one CUDA graph (integrate -> narrowphase -> resolve
per frame).  The metric is body-steps/s = bodies x frames / time.

  value       precision form (float32 bulk, float64 islands) with the learned
              warm start of adjustVelocities (network trained before timing,
              on the GPU, on contacts harvested from scenes of other seeds),
              device time of the rollout graph (CUDA events recorded on the
              batch stream inside the graph), inputs resident in HBM
  e2e         the same through the C ABI with host buffers: cz_upload_bodies
              (host -> device) + cz_step + cz_download_bodies (device -> host)
  fp32_plain  the precision form without the warm start, measured the same way
  fp64        the plain float64 form measured the same way (reported beside it)
  accuracy    both precision variants against the float64 form
  roofline    the dominant kernel, algorithmic bytes per launch / its average
              CUDA-event duration over the timed rollouts
  cpu_baseline  the oracle (C++ restatement of the reference's float64 Go path)
              on the host's cores, one thread per world, on a bounded sample

--workload piles measures the large-world configuration instead: 256 worlds x
1024 cubes (16 x 16 x 4 lattice, dropped 0.5 m), 300 frames, float32 and
float64 forms; metric pair-tests/s (ordered narrowphase pair and half-space
tests per second over the narrowphase time) with body-steps/s beside it.  The
learned warm start serves worlds within the resolver's shared-memory slot
only, so the large worlds run the plain precision form.

--impl reference times the reference's CPU path (the oracle port; the Go
reference cannot be built here) on all host cores with the same metric; with
--workload piles, the ordered narrowphase of one pile world per host thread,
in pair-tests/s.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "body-steps/s: FP32+MLP warm-start vs plain FP64 on 1 GB300 at stated error"
UNIT = "body-steps/s"
DT = 1.0 / 60.0
L2_BYTES = 126 * 1024 * 1024
# DRAM bytes (read + write) of one resolver launch at steady state on the
# default workload (16384 worlds x 32 bodies), per form, from an ncu capture
# of the resolver instantiation that form runs (frame 381 of a 400-frame
# rollout): the roofline's measured traffic beside its algorithmic bytes.
RESOLVE_TRAFFIC = {
    "fp32_mlp": {"bytes": 255.9e6, "kernel": "k_resolve<float, double, 32, true>",
                 "source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch"},
}


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.out = None

    def __enter__(self):
        try:
            self.out = open(os.path.join("/tmp", "cz_clocks_%d.csv" % os.getpid()), "w+")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.out,
                                         stderr=subprocess.DEVNULL)
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

    def summary(self):
        if self.out is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.out.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out.read().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        load = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": float(np.median(load)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def _flush_l2():
    import torch
    buf = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    buf.fill_(1.0)
    torch.cuda.synchronize()
    del buf


def _kinetic_energy(d, scene):
    inv_m = scene.inverse_mass
    v = d["velocity"]
    w = d["rotation"]
    iw = d["inverse_inertia_world"].reshape(-1, 3, 3).transpose(0, 2, 1)  # column-major -> row-major
    lin = 0.5 * np.einsum("ij,ij->i", v, v) / inv_m
    iw_inv = np.linalg.inv(iw)
    ang = 0.5 * np.einsum("ij,ijk,ik->i", w, iw_inv, w)
    return lin + ang


def accuracy(scene, frames, batches, forms=("fp32_mlp", "fp32")):
    """Errors of the precision variants against the plain float64 form
    (bit-exact with the oracle) on identical initial states: one-step
    relative error per quantity (per body, max-norm error over max(|value|, 1)),
    time-averaged kinetic energy and final mean height."""
    res = {}
    for name, b in batches.items():
        b.restore()
        b.step(1, DT)
        res[name] = b.download()
    ke = {name: [] for name in batches}
    height = {}
    seg = 30
    for name, b in batches.items():
        b.restore()
        for s in range(0, frames, seg):
            b.step(min(seg, frames - s), DT)
            d = b.download()
            ke[name].append(float(_kinetic_energy(d, scene).sum()))
        height[name] = float(d["position"][:, 1].mean())
    out = {"mean_height_fp64_m": height["fp64"], "ke_time_avg_fp64_J": float(np.mean(ke["fp64"]))}
    r = res["fp64"]
    for f in forms:
        if f not in batches:
            continue
        a = res[f]
        one = {}
        for k in ("position", "orientation", "velocity", "rotation"):
            den = np.maximum(np.abs(r[k]).max(axis=1), 1.0)
            e = np.abs(a[k] - r[k]).max(axis=1) / den
            one[k] = {"max": float(e.max()), "p99": float(np.quantile(e, 0.99)),
                      "frac_le_1e-4": float((e <= 1e-4).mean())}
        out[f] = {"one_step_rel_error": one,
                  "ke_time_avg_rel_diff": float(abs(np.mean(ke[f]) - np.mean(ke["fp64"])) / np.mean(ke["fp64"])),
                  "mean_height_rel_diff": float(abs(height[f] - height["fp64"]) / abs(height["fp64"]))}
    return out


def _alg_bytes(phase, real, nbodies, counters, frames, rollouts):
    """Algorithmic HBM bytes per launch of a phase (the minimum each kernel must move)."""
    launches = frames * rollouts
    contacts = counters["contacts"] / launches
    resolved = counters["contacts_resolved"] / launches
    if phase == 0:  # integrate: 13 state reals read and written, a symmetric inverse inertia (6) read and one written
        return nbodies * 38 * real
    if phase == 1:  # narrowphase: stage 11 rows + shape, write contacts (9 reals + packed bodies)
        return nbodies * (11 * real + 4) + contacts * (9 * real + 4)
    # resolver: bodies in (27 reals + flag) and out (23 reals + flag), contacts in
    return nbodies * (50 * real + 2) + resolved * (9 * real + 4)


def run_ours(args):
    import torch
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from cubez_gb300 import _lib, scenes
    from cubez_gb300.batch import FORM_FP32, FORM_FP64, WorldBatch

    scene = scenes.precision(num_worlds=args.worlds, bodies=args.bodies, seed=3 + 1000 * rank)
    nb = scene.num_bodies
    frames = args.frames

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    from cubez_gb300 import autotune, learned
    forms = [("fp32_mlp", FORM_FP32), ("fp32", FORM_FP32), ("fp64", FORM_FP64)]
    if args.fp32_only:
        forms = forms[:2]
    if args.forms:
        forms = [f for f in forms if f[0] in args.forms.split(",")]
    train_info = None
    if any(name == "fp32_mlp" for name, _ in forms):
        t0 = time.perf_counter()
        blob, train_info = learned.train_warm_start(num_worlds=args.train_worlds, device=local)
        train_info["seconds"] = time.perf_counter() - t0
    fixed = json.loads(args.tuning) if args.tuning else None
    batches = {}
    tuning = {}
    for name, form in forms:
        b = WorldBatch.from_scene(scene, form=form, device=local)
        if name == "fp32_mlp":
            learned.set_warm_start(b, blob)
        if fixed:
            b.set_tuning(**fixed)
            tuning[name] = b.get_tuning()
        elif args.autotune:
            # tune on a settled state (half-way through the rollout), untimed
            b.step(frames // 2, DT)
            b.snapshot()
            cfg, _ = autotune.tune(b, frames=args.tune_frames, dt=DT)
            tuning[name] = cfg
            b.upload(scene)
        b.prepare_rollout(frames, DT)  # damping factors + graph capture, outside any timed region
        b.snapshot()
        batches[name] = b

    results = {}
    for name, _ in forms:
        b = batches[name]
        # the float64 comparison form takes ~30 s per rollout: one warm-up and
        # one timed rollout unless asked otherwise
        warmup, steps = (args.fp64_warmup, args.fp64_steps) if name == "fp64" else (args.warmup, args.steps)
        for _ in range(warmup):
            b.restore()
            b.step_timed(frames, DT)
        b.counters(reset=True)
        tot_ms, ph_ms = 0.0, np.zeros(3)
        launches0 = _lib.kernel_launches()
        clocks = Clocks(local)
        with clocks:
            for _ in range(steps):
                b.restore()
                _flush_l2()
                barrier()
                t, ph = b.step_timed(frames, DT)
                barrier()
                tot_ms += t
                ph_ms += ph
        launches = _lib.kernel_launches() - launches0
        cnt = b.counters()
        ms = tot_ms / steps
        if ws > 1:
            import torch.distributed as dist
            tt = torch.tensor([ms], device="cuda")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            ms = float(tt.item())
        results[name] = {"ms_per_step": ms, "phase_ms": (ph_ms / steps).tolist(), "counters": cnt,
                         "launches": launches, "clocks": clocks.summary(), "steps": steps, "warmup": warmup,
                         "value": nb * frames * ws / (ms / 1e3)}

    head = "fp32_mlp" if "fp32_mlp" in results else forms[0][0]
    # e2e through the C ABI with host buffers (the headline form)
    e2e = None
    if not args.no_e2e:
        b = batches[head]
        host = {k: np.ascontiguousarray(getattr(scene, k)) for k in scene.FIELDS}
        import ctypes as C
        pinned = {}
        for k, v in host.items():
            t = torch.empty(v.nbytes, dtype=torch.uint8, pin_memory=True)
            a = np.frombuffer(t.numpy().data, dtype=v.dtype, count=v.size).reshape(v.shape)
            a[...] = v
            pinned[k] = (t, a)
        arrays = {k: a for k, (t, a) in pinned.items()}
        for _ in range(max(1, args.warmup)):
            b.upload(**arrays)
            b.step(frames, DT)
            b.download()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            b.upload(**arrays)
            b.step(frames, DT)
            out = b.download()
        barrier()
        e2e_s = (time.perf_counter() - t0) / args.steps
        real_h2d = 43 * 8 * nb + 2 * nb + 4 * nb + 2 * 8 * int(b.info()["padded_bodies"])
        real_d2h = 43 * 8 * nb + 2 * nb + 4 * nb + 4
        e2e = {"value": nb * frames * ws / e2e_s, "unit": UNIT, "h2d_bytes_per_step": real_h2d,
               "d2h_bytes_per_step": real_d2h, "ms_per_step": e2e_s * 1e3}
        del C, out

    acc = accuracy(scene, frames, batches) if not args.no_accuracy and "fp64" in batches else None

    r32 = results[head]
    real = 4 if batches[head].form == FORM_FP32 else 8
    default_size = args.worlds == 16384 and args.bodies == 32 and real == 4
    phase_names = ["integrate", "narrowphase", "resolve"]
    ph = r32["phase_ms"]
    # the fused frame (tuning fused_frame 1) reports its whole time as the resolve phase
    fused = ph[0] == 0.0 and ph[1] == 0.0
    if fused:
        phase_names[2] = "frame"
    dom = int(np.argmax(ph))
    per_launch_ms = ph[dom] / frames
    alg = [_alg_bytes(i, real, nb, r32["counters"], frames, args.steps) for i in range(3)]
    bytes_launch = sum(alg) if fused else alg[dom]
    peak, peak_kind = _peaks()
    achieved = bytes_launch / (per_launch_ms / 1e3) / 1e9
    kernels = {}
    for i, n in enumerate(phase_names):
        if fused and i < 2:
            continue
        bl = sum(alg) if fused else alg[i]
        pl = ph[i] / frames
        kernels[n] = {"ms_per_launch": pl, "share": ph[i] / sum(ph), "alg_bytes_per_launch": bl,
                      "gbs": bl / (pl / 1e3) / 1e9}
        if i == 0:  # what the kernel moves: 37 reals + 2 flag bytes read, 25 reals written
            kernels[n]["moved_bytes_per_launch"] = nb * (62 * real + 2)
            kernels[n]["moved_gbs"] = nb * (62 * real + 2) / (pl / 1e3) / 1e9
    traffic = RESOLVE_TRAFFIC.get(head) if default_size and dom == 2 and not fused else None
    info = batches[head].info()
    for b in batches.values():
        b.close()

    if rank != 0:
        return
    cpu = None if args.no_cpu_baseline else cpu_baseline(args, scene)
    secondary = None if (args.no_secondary or ws > 1) else secondary_samples(local)
    def block(name):
        if name not in results:
            return None
        r = results[name]
        return {"value": r["value"], "ms_per_step": r["ms_per_step"], "phase_ms": r["phase_ms"],
                "steps": r["steps"], "warmup": r["warmup"], "clocks": r["clocks"], "gpu_launches": r["launches"],
                "counters_per_frame": {k: v / (frames * r["steps"]) for k, v in r["counters"].items()}}

    fp64v = results["fp64"]["value"] if "fp64" in results else None
    cnt = r32["counters"]
    line = {
        "metric": METRIC, "value": r32["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r32["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (f64 islands) + bf16 MLP", "data": "synthetic (seeded scenes)",
        "config": {"workload": "precision: %d worlds x %d bodies (16 spheres + 16 cubes), %d-frame rollout, "
                               "dt=1/60, iterations 4 x contacts" % (args.worlds, args.bodies, frames),
                   "form": {"fp32_mlp": "fp32 + learned warm start (18-64-64-64-3 BF16 MLP on tensor cores)",
                            "fp32": "fp32 (f64 islands), plain resolver", "fp64": "fp64, bit-exact"}[head],
                   "step": "one %d-frame rollout" % frames,
                   "l2": "explicit 252 MB flush before every timed rollout; working set > L2",
                   "parallelism": "weak: %d worlds per GPU" % args.worlds},
        "fp32_plain": block("fp32"),
        "fp64": block("fp64"),
        "mlp_over_fp64": (r32["value"] / fp64v) if fp64v and head == "fp32_mlp" else None,
        "fp32_plain_over_fp64": (results["fp32"]["value"] / fp64v) if fp64v and "fp32" in results else None,
        "mlp_over_fp32_plain": (r32["value"] / results["fp32"]["value"]) if "fp32" in results else None,
        "warm_start": None if train_info is None else {"training": train_info,
                       "policy": "worlds whose previous solve used at most 1/%d of the iteration budget are "
                                 "warm-started (warm_start_budget_shift %d); the tuner does not change it"
                                 % (1 << tuning.get("fp32_mlp", {}).get("warm_start_budget_shift", 2),
                                    tuning.get("fp32_mlp", {}).get("warm_start_budget_shift", 2)),
                       "warm_worlds_per_frame": cnt["warm_worlds"] / (frames * args.steps),
                       "warm_bodies_per_frame": cnt["warm_bodies"] / (frames * args.steps),
                       "mean_scale": cnt["warm_scale_sum"] / max(1, cnt["warm_bodies"]),
                       "fallbacks_per_frame": cnt["warm_fallbacks"] / (frames * args.steps),
                       "vel_iterations_vs_plain": cnt["vel_iterations"] / max(
                           1, results["fp32"]["counters"]["vel_iterations"]) if "fp32" in results else None},
        "accuracy": acc,
        "e2e": e2e,
        "gpu_launches": r32["launches"],
        "clocks": r32["clocks"],
        "roofline": {"kernel": phase_names[dom], "bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": traffic["bytes"] if traffic else None,
                     "traffic_source": dict(traffic, bytes=None) if traffic else None,
                     "note": "the resolver is sequential per world and latency / float64-pipe bound; its HBM "
                             "fraction is reported as asked, iterations per second below"},
        "resolver_iterations_per_s": (cnt["pos_iterations"] + cnt["vel_iterations"]) / (args.steps * ph[2] / 1e3),
        "kernels": kernels,
        "counters_per_frame": {k: v / (frames * args.steps) for k, v in cnt.items()},
        "batch": info,
        "tuning": tuning,
        "cpu_baseline": cpu,
        "secondary": secondary,
    }
    print(json.dumps(line))


def _sample_rollout(scene, form, frames, local, units=None, warmup=1):
    """`warmup` untimed rollouts and one timed rollout of `frames` frames
    (default tuning): body-steps/s, and pair-tests/s of the narrowphase when
    `units` (tests per frame) is given."""
    import torch
    from cubez_gb300.batch import WorldBatch
    b = WorldBatch.from_scene(scene, form=form, device=local)
    b.prepare_rollout(frames, DT)  # the graph capture, untimed
    b.snapshot()
    for _ in range(warmup):
        b.step_timed(frames, DT)
        b.restore()
    _flush_l2()
    clocks = Clocks(local)
    with clocks:
        torch.cuda.synchronize()
        tot, ph = b.step_timed(frames, DT)
    b.close()
    r = {"ms_per_step": tot, "phase_ms": [float(x) for x in ph], "clocks": clocks.summary(),
         "body_steps_per_s": scene.num_bodies * frames / (tot / 1e3)}
    if units is not None:
        r["pair_tests_per_s"] = units * frames / (ph[1] / 1e3)
    return r


def secondary_samples(local):
    """One rollout of each secondary configuration at its full size, so that
    the default run records them too (default tuning, one timed rollout; the
    tuned runs with more steps: --workload piles / batched): 64 cube piles of
    1024 bodies over 60 frames in both forms, and the batched float64 worlds
    (4096 x U{8..64}) over 600 frames."""
    from cubez_gb300 import scenes
    from cubez_gb300.batch import FORM_FP32, FORM_FP64
    piles = scenes.piles(num_worlds=64, seed=5)
    n = int(piles.counts[0])
    units = piles.num_worlds * (n * (n - 1) + n)
    out = {"piles": {"workload": "64 worlds x %d cubes, 60 frames, default tuning, one timed rollout per form" % n,
                     "fp32": _sample_rollout(piles, FORM_FP32, 60, local, units),
                     "fp64": _sample_rollout(piles, FORM_FP64, 60, local, units, warmup=0)}}
    mixed = scenes.mixed(num_worlds=4096, seed=2)
    out["batched_fp64"] = {"workload": "4096 worlds x U{8..64} (%d bodies), 600 frames, float64, default tuning, "
                                       "one timed rollout" % mixed.num_bodies,
                           "fp64": _sample_rollout(mixed, FORM_FP64, 600, local, warmup=0)}
    return out


def cpu_baseline(args, scene):
    """The oracle (C++ restatement of the reference's float64 path), one
    thread per world on all host cores, on the first `cpu_worlds` worlds."""
    from oracle.oracle import OracleBatch, hardware_threads
    cores = os.cpu_count() or hardware_threads()
    nw = min(args.cpu_worlds, scene.num_worlds)
    sub = scene.subset(range(nw))
    ob = OracleBatch(sub)
    t0 = time.perf_counter()
    ob.step(args.frames, DT, 4, cores)
    el = time.perf_counter() - t0
    return {"value": sub.num_bodies * args.frames / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d of %d worlds x %d frames (float64 oracle, %.1f s)" % (nw, scene.num_worlds, args.frames, el)}


def run_reference_piles(args):
    """The large-world metric (narrowphase pair-tests/s) on the oracle: the
    ordered all-pairs narrowphase of a sample of pile worlds, one world per
    host thread (each world its own oracle batch; the calls release the GIL)."""
    from concurrent.futures import ThreadPoolExecutor

    from cubez_gb300 import scenes
    from oracle.oracle import OracleBatch, hardware_threads
    cores = os.cpu_count() or hardware_threads()
    nw = args.worlds if args.worlds != 16384 else 256
    sample = min(nw, cores)
    scene = scenes.piles(num_worlds=nw, seed=5)
    n = int(scene.counts[0])
    units = sample * (n * (n - 1) + n)
    batches = [OracleBatch(scene.subset([w])) for w in range(sample)]
    for ob in batches:
        ob.integrate(DT)
    total = 0.0
    with ThreadPoolExecutor(cores) as ex:
        for _ in range(args.warmup):
            list(ex.map(lambda ob: ob.narrowphase(), batches))
        for _ in range(args.steps):
            t0 = time.perf_counter()
            list(ex.map(lambda ob: ob.narrowphase(), batches))
            total += time.perf_counter() - t0
    value = units * args.steps / total
    line = {"metric": "pair-tests/s (large worlds, secondary)", "value": value, "unit": "pair-tests/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded scenes)", "impl": "reference",
            "config": {"workload": "piles: %d worlds x %d cubes; each step the narrowphase of %d worlds" %
                                   (nw, n, sample), "parallelism": "host cores, one thread per world"},
            "cpu_baseline": {"value": value, "unit": "pair-tests/s", "cores": cores, "kind": "port",
                             "sample": "%d of %d worlds, first frame (the Go reference cannot be built here; its "
                                       "float64 path restated in C++)" % (sample, nw)},
            "e2e": {"value": value, "unit": "pair-tests/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    if args.workload == "piles":
        run_reference_piles(args)
        return
    from cubez_gb300 import scenes
    from oracle.oracle import OracleBatch, hardware_threads
    batched = args.workload == "batched"
    if batched:
        scene = scenes.mixed(num_worlds=args.worlds if args.worlds != 16384 else 4096, seed=2)
    else:
        scene = scenes.precision(num_worlds=args.worlds, bodies=args.bodies, seed=3)
    cores = os.cpu_count() or hardware_threads()
    nw = min(args.cpu_worlds, scene.num_worlds)
    sub = scene.subset(range(nw))
    for _ in range(args.warmup):
        OracleBatch(sub).step(min(args.frames, 30), DT, 4, cores)
    total = 0.0
    for _ in range(args.steps):
        ob = OracleBatch(sub)
        t0 = time.perf_counter()
        ob.step(args.frames, DT, 4, cores)
        total += time.perf_counter() - t0
    ms = total / args.steps * 1e3
    value = sub.num_bodies * args.frames / (ms / 1e3)
    line = {
        "metric": "body-steps/s (batched float64, secondary)" if batched else METRIC, "value": value, "unit": UNIT,
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded scenes)", "impl": "reference",
        "config": {"workload": ("batched: %d worlds x U{8..64} spheres/cubes, %d-frame rollout, dt=1/60, float64; "
                                "each step a sample of %d worlds" % (scene.num_worlds, args.frames, nw)) if batched else
                               ("precision: %d worlds x %d bodies, %d-frame rollout, dt=1/60; each step a sample of "
                                "%d worlds" % (args.worlds, args.bodies, args.frames, nw)),
                   "parallelism": "host cores, one thread per world"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "%d of %d worlds x %d frames per step (the Go reference cannot be built here; "
                                   "its float64 path restated in C++)" % (nw, scene.num_worlds, args.frames)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_piles(args):
    """The large-world configuration: bounded timing (one rollout per form
    after an untimed warm-up of `--warmup` rollouts, default 0 here: one
    float64 rollout takes minutes), a CPU sample of one world."""
    import torch
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    from cubez_gb300 import _lib, scenes
    from cubez_gb300.batch import FORM_FP32, FORM_FP64, WorldBatch
    nw = args.worlds if args.worlds != 16384 else 256
    frames = args.frames if args.frames != 600 else 300
    scene = scenes.piles(num_worlds=nw, seed=5 + 1000 * rank)
    n = int(scene.counts[0])
    units = nw * (n * (n - 1) + n)  # ordered pair tests + half-space tests per frame
    out = {}
    settled = None
    fixed = json.loads(args.tuning) if args.tuning else None
    for name, form in (("fp32", FORM_FP32), ("fp64", FORM_FP64)):
        b = WorldBatch.from_scene(scene, form=form, device=local)
        if fixed:
            b.set_tuning(**fixed)
        b.prepare_rollout(frames, DT)
        b.snapshot()
        for _ in range(args.warmup if args.warmup_given else 0):
            b.restore()
            b.step_timed(frames, DT)
        b.restore()
        b.counters(reset=True)
        launches0 = _lib.kernel_launches()
        clocks = Clocks(local)
        with clocks:
            torch.cuda.synchronize()
            tot, ph = b.step_timed(frames, DT)
        cnt = b.counters()
        out[name] = {"ms_per_step": tot, "phase_ms": [float(p) for p in ph], "clocks": clocks.summary(),
                     "gpu_launches": _lib.kernel_launches() - launches0,
                     "body_steps_per_s": scene.num_bodies * frames / (tot / 1e3),
                     "pair_tests_per_s": units * frames / (ph[1] / 1e3),
                     "counters_per_world_frame": {k: v / (frames * nw) for k, v in cnt.items()}}
        if name == "fp64":
            settled = b.download(("position", "orientation", "velocity", "rotation"))
        b.close()
    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        # one world, 10 frames from the float64 state after the rollout (piles at rest)
        from oracle.oracle import OracleBatch
        one = scene.subset([0])
        for k, v in settled.items():
            setattr(one, k, v[:n])
        ob = OracleBatch(one)
        t0 = time.perf_counter()
        ob.step(10, DT, 4, 1)
        el = time.perf_counter() - t0
        cpu = {"value": n * 10 / el, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "1 world x 10 frames from the settled float64 state (float64 oracle, %.1f s)" % el}
    if rank != 0:
        return
    r = out["fp32"]
    line = {"metric": "pair-tests/s (large worlds, secondary)", "value": r["pair_tests_per_s"], "unit": "pair-tests/s",
            "n_gpus": ws, "steps": 1, "warmup": args.warmup if args.warmup_given else 0,
            "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (f64 islands)", "data": "synthetic (seeded scenes)",
            "config": {"workload": "piles: %d worlds x %d cubes (16x16x4 lattice, dropped 0.5 m), %d frames, dt=1/60"
                                   % (nw, n, frames), "step": "one %d-frame rollout" % frames},
            "body_steps_per_s": r["body_steps_per_s"], "fp32": r, "fp64": out["fp64"],
            "fp32_over_fp64": r["body_steps_per_s"] / out["fp64"]["body_steps_per_s"],
            "gpu_launches": r["gpu_launches"], "clocks": r["clocks"], "cpu_baseline": cpu}
    print(json.dumps(line))


def run_batched(args):
    """The batched configuration: 4096 worlds of U{8..64} spheres and cubes in
    the plain float64 form (bit-exact with the reference's arithmetic), one
    600-frame rollout per step captured as one CUDA graph, restarted from the
    same device-resident state; e2e through the C ABI with host buffers; the
    oracle on the host's cores beside it."""
    import torch
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from cubez_gb300 import _lib, scenes
    from cubez_gb300.batch import FORM_FP64, WorldBatch
    nw = args.worlds if args.worlds != 16384 else 4096
    frames = args.frames
    scene = scenes.mixed(num_worlds=nw, seed=2 + 1000 * rank)
    nb = scene.num_bodies
    b = WorldBatch.from_scene(scene, form=FORM_FP64, device=local)
    fixed = json.loads(args.tuning) if args.tuning else None
    if fixed:
        b.set_tuning(**fixed)
    elif args.autotune:
        from cubez_gb300 import autotune
        # tune on a settled state (half-way through the rollout), untimed
        b.step(frames // 2, DT)
        b.snapshot()
        autotune.tune(b, frames=args.tune_frames, dt=DT)
        b.upload(scene)
    tuning = b.get_tuning()
    b.prepare_rollout(frames, DT)
    b.snapshot()

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        b.restore()
        b.step_timed(frames, DT)
    b.counters(reset=True)
    launches0 = _lib.kernel_launches()
    tot, ph = 0.0, np.zeros(3)
    clocks = Clocks(local)
    with clocks:
        for _ in range(args.steps):
            b.restore()
            _flush_l2()
            barrier()
            t, p = b.step_timed(frames, DT)
            barrier()
            tot += t
            ph += p
    launches = _lib.kernel_launches() - launches0
    cnt = b.counters()
    ms = tot / args.steps
    if ws > 1:
        import torch.distributed as dist
        tt = torch.tensor([ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    # e2e: upload from pinned host memory, the rollout, download
    e2e = None
    if not args.no_e2e:
        pinned = {}
        for k in scene.FIELDS:
            v = np.ascontiguousarray(getattr(scene, k))
            t = torch.empty(v.nbytes, dtype=torch.uint8, pin_memory=True)
            a = np.frombuffer(t.numpy().data, dtype=v.dtype, count=v.size).reshape(v.shape)
            a[...] = v
            pinned[k] = (t, a)
        arrays = {k: a for k, (t, a) in pinned.items()}
        b.upload(**arrays)
        b.step(frames, DT)
        b.download()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            b.upload(**arrays)
            b.step(frames, DT)
            b.download()
        barrier()
        e2e_s = (time.perf_counter() - t0) / args.steps
        h2d = 43 * 8 * nb + 2 * nb + 4 * nb + 2 * 8 * int(b.info()["padded_bodies"])
        d2h = 43 * 8 * nb + 2 * nb + 4 * nb + 4
        e2e = {"value": nb * frames * ws / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "ms_per_step": e2e_s * 1e3}
    info = b.info()
    b.close()
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        from oracle.oracle import OracleBatch, hardware_threads
        cores = os.cpu_count() or hardware_threads()
        sub = scene.subset(range(min(args.cpu_worlds, nw)))
        ob = OracleBatch(sub)
        t0 = time.perf_counter()
        ob.step(frames, DT, 4, cores)
        el = time.perf_counter() - t0
        cpu = {"value": sub.num_bodies * frames / el, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "%d of %d worlds x %d frames (float64 oracle, %.1f s)" % (sub.num_worlds, nw, frames, el)}
    per = {k: v / (frames * args.steps) for k, v in cnt.items()}
    line = {"metric": "body-steps/s (batched float64, secondary)", "value": nb * frames * ws / (ms / 1e3),
            "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded scenes)",
            "config": {"workload": "batched: %d worlds x U{8..64} spheres/cubes (%d bodies), %d-frame rollout, "
                                   "dt=1/60, float64" % (nw, nb, frames), "step": "one %d-frame rollout" % frames,
                       "l2": "explicit 252 MB flush before every timed rollout"},
            "world_steps_per_s": nw * frames * ws / (ms / 1e3), "phase_ms": (ph / args.steps).tolist(),
            "counters_per_frame": per, "gpu_launches": launches, "clocks": clocks.summary(), "e2e": e2e,
            "batch": info, "tuning": tuning, "cpu_baseline": cpu}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--worlds", type=int, default=16384)
    ap.add_argument("--bodies", type=int, default=32)
    ap.add_argument("--frames", type=int, default=600)
    ap.add_argument("--cpu-worlds", type=int, default=2048)
    ap.add_argument("--train-worlds", type=int, default=4096)
    ap.add_argument("--workload", default="precision", choices=["precision", "piles", "batched"])
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--fp64-warmup", type=int, default=1)
    ap.add_argument("--fp32-only", action="store_true")
    ap.add_argument("--forms", default="", help="comma-separated subset of fp32_mlp,fp32,fp64")
    ap.add_argument("--tuning", default="", help="fixed tuning knobs as JSON (skips the autotuner)")
    ap.add_argument("--autotune", type=int, default=1)
    ap.add_argument("--tune-frames", type=int, default=30)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true", help="skip the short piles / batched samples")
    args = ap.parse_args()
    import sys as _sys
    args.warmup_given = any(a.startswith("--warmup") for a in _sys.argv[1:])
    if args.workload == "piles" and args.impl != "reference":
        run_piles(args)
    elif args.workload == "batched" and args.impl != "reference":
        run_batched(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
