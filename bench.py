#!/usr/bin/env python3
"""Benchmark: meshify (smooth + marching cubes + weld) of the 512^3 CT-like
workload on GB300, in Gvox/s.

Workload: 512^3 float32, background N(-1000,20), 300 ellipsoidal structures,
1% salt noise at +2000, iso 300, -p 1 -l 0 -b 0 -o 0 (Lewiner MC33) -r 1 -s 0.
A step = one full meshify of that volume (pre-smooth, range, bbox, marching
cubes count + emit, weld, degenerate removal) with the volume resident in HBM
(537 MB > 129 MB L2, so no L2 flush is needed between steps).  `e2e` measures
the same through the C ABI with host buffers: the volume is copied from pinned
host memory and the mesh (vec3d/vec3i) copied back every step.

--impl reference times the reference algorithm on the host cores: the CPU
oracle port (the reference's C path restated), or the reference itself when
oracle/_ref was built on this machine.

Multi-GPU: the path does not shard across GPUs in this build (replicas only):
each rank meshes its own copy and `value` counts the voxels of all ranks.
"""
import argparse
import json

import numpy as np
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Gvox/s smooth+MC+weld at 512³; atlas meshes/s batched vs loop; fwd+bwd ms @128³"
WORKLOAD = "ct512: 512^3 f32 CT-like, iso 300, -p 1 -l 0 -b 0 -o 0 -r 1 -s 0 (Lewiner MC33)"
ISO = 300.0
# DRAM bytes (read + write) per step of each stage on this workload: one ncu capture of
# `bench.py --profile 384` (dram__bytes_read.sum + dram__bytes_write.sum of the stage's kernels),
# scaled by the voxel count to 512^3 (profiles/meshify_ct512_kernels.md): smooth = pass A + pass B,
# count = signs, marks, exact passes on marked voxels, words, scans, emit = k_emit, weld, degenerate
SCALE_384 = (512 / 384) ** 3
NCU_TRAFFIC = {"smooth": 437.9e6 * SCALE_384, "count": 654.6e6 * SCALE_384, "emit": 138.0e6 * SCALE_384,
               "weld": 74.0e6 * SCALE_384, "degenerate": 125.6e6 * SCALE_384}
PASS_A_TRAFFIC = 437.6e6 * SCALE_384   # k_od_approx alone
# what bounds each stage (measured in the same profiles)
STAGE_BOUND = {"smooth": "FP32 instruction issue in pass A (74 % issue active, ~92 instructions per voxel); "
                         "DRAM 7.7 B/voxel, no re-reads",
               "count": "the exact passes on the ~10 % marked voxels (issue + sector-granular gathers) and the "
                        "sign/word passes",
               "emit": "latency (neighbour-word and value loads) and divergent listing"}
STAGE_NAMES = ("smooth", "cluster", "count", "emit", "weld", "degenerate", "hc")


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.proc, self.file = index, None, None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().strip().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
                for n, v in zip(names, r[4:8]):
                    if "Active" in v and "Not" not in v:
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def slowest_rank_ms(ms, dist, device=None):
    """The job's time: the maximum over ranks of each rank's timed-region
    milliseconds (replicas: every rank meshes its own copy of the workload).
    Works on NCCL (CUDA tensor) and gloo (CPU tensor) process groups."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(units_per_rank, world, ms):
    """Whole-job throughput: units of all ranks over the slowest rank's time, in G units/s."""
    return world * units_per_rank / (ms * 1e-3) / 1e9


def dist_setup(n):
    import torch
    if n <= 1:
        return 0, 1, None
    import torch.distributed as dist
    rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl", init_method="env://")
    return rank, world, dist


def cpu_reference(vol, steps, warmup):
    """Time the reference algorithm on the host (one thread: meshify is serial)."""
    from oracle.oracle import Oracle, Reference, reference_available
    if reference_available():
        impl, kind = Reference(False), "reference"
    else:
        impl, kind = Oracle(), "port"
    times = []
    for i in range(warmup + steps):
        t0 = time.perf_counter()
        m = impl.meshify(vol, ISO, 0, True, False, False)
        t1 = time.perf_counter()
        if i >= warmup:
            times.append(t1 - t0)
    assert m is not None
    nvox = vol.size
    return nvox / statistics.median(times) / 1e9, kind, times, m


def _reference_worker(path, rounds, start, done, out):
    """one host core: meshify the volume at `path` once per round, in step with the others"""
    from oracle.oracle import Oracle, Reference, reference_available
    impl = Reference(False) if reference_available() else Oracle()
    vol = np.load(path)
    for _ in range(rounds):
        start.wait()
        m = impl.meshify(vol, ISO, 0, True, False, False)
        out.put((0, 0) if m is None else (len(m[0]), len(m[1])))
        done.wait()


def _atlas_worker(path, label, start, out):
    """one host core: the reference's per-label atlas work for one label"""
    from oracle.oracle import Oracle
    o = Oracle()
    img = np.load(path).astype(np.float32)
    start.wait()
    b, _ = o.binarize_label(img, label)
    m = o.meshify(b, 0.5, 0, True, True, True)
    if m is not None:
        o.laplacian_smoothHC(m[1], m[0], 0.1, 0.5, 5, True)
    out.put(label)


def cpu_reference_parallel(vol, steps, warmup, procs):
    """The reference algorithm on `procs` host cores at once: meshify is
    single-threaded, so each core meshes its own copy of the volume and a step
    is the wall time until all of them are done (procs volumes per step)."""
    import multiprocessing as mp
    from oracle.oracle import reference_available
    kind = "reference" if reference_available() else "port"
    tmp = tempfile.mkdtemp(prefix="n2m_ref_", dir="/dev/shm" if os.path.isdir("/dev/shm") else None)
    path = os.path.join(tmp, "vol.npy")
    np.save(path, vol)
    ctx = mp.get_context("spawn")
    start, done, out = ctx.Barrier(procs + 1), ctx.Barrier(procs + 1), ctx.Queue()
    rounds = warmup + steps
    ws = [ctx.Process(target=_reference_worker, args=(path, rounds, start, done, out), daemon=True)
          for _ in range(procs)]
    for w in ws:
        w.start()
    times, counts = [], (0, 0)
    try:
        for i in range(rounds):
            start.wait(timeout=600)
            t0 = time.perf_counter()
            res = [out.get(timeout=600) for _ in range(procs)]
            t1 = time.perf_counter()
            done.wait(timeout=600)
            assert all(r[0] > 0 for r in res)
            counts = res[0]
            if i >= warmup:
                times.append(t1 - t0)
    finally:
        for w in ws:
            w.join(timeout=60)
        os.remove(path)
        os.rmdir(tmp)
    return procs * vol.size / statistics.median(times) / 1e9, kind, times, counts


def host_procs(bytes_per_proc=4.5e9):
    """host cores for concurrent reference runs, bounded by the memory each run needs"""
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    avail = None
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    avail = int(line.split()[1]) * 1024
    except OSError:
        pass
    if avail is None:
        return 1
    return max(1, min(cores, int(0.6 * avail / bytes_per_proc)))


GD_LR = 4.0   # Adam step on the voxel intensities (the spheres are 100 on 0, iso 50)


def adjoint_metric(n2m, torch, steps=20, gd_steps=200):
    """fwd and fwd+bwd ms on the 128^3 differentiation workload (pre-smooth,
    Lewiner MC, 10 HC iterations; loss = sum(|v - c| - 40)^2), the gradient's
    error against the FP64 host gradient of the same map, and 200 steps of
    shape fitting (Adam on the voxel intensities; the mesh and its topology are
    recomputed every step)."""
    from nii2mesh_gb300 import synth
    from nii2mesh_gb300.autograd import MeshifyFunction, sphere_loss
    ctx = n2m.Context(torch.cuda.current_device())
    host = synth.sphere128()
    img = torch.from_numpy(host).cuda()
    center, radius = (63.5, 63.5, 63.5), 40.0
    nvox = host.size

    def fwd(v):
        pts, _ = MeshifyFunction.apply(v, ctx, 50.0, 10)
        return sphere_loss(pts, center, radius)

    def timed(fn, n):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(n):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / n * 1e3

    def f_only():
        with torch.no_grad():
            float(fwd(img))

    def f_b():
        v = img.clone().requires_grad_(True)
        fwd(v).backward()
        return v.grad

    t_f = timed(f_only, steps)
    t_fb = timed(f_b, steps)
    grad = f_b().cpu().numpy()
    # shape fitting: the loss is read back only at the first and the last step.  One untimed step
    # first: the first optimizer step of a process compiles and caches torch's kernels for this GPU
    w_ = img.clone().requires_grad_(True)
    o_ = torch.optim.Adam([w_], lr=GD_LR)
    fwd(w_).backward()
    o_.step()
    torch.cuda.synchronize()
    del w_, o_
    v = img.clone().requires_grad_(True)
    opt = torch.optim.Adam([v], lr=GD_LR)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    first = last = None
    for it in range(gd_steps):
        opt.zero_grad(set_to_none=True)
        loss = fwd(v)
        loss.backward()
        opt.step()
        if it == 0:
            first = loss.detach()
        last = loss.detach()
        torch.cuda.synchronize()   # one fitting step at a time, as a loop that inspects each mesh runs
    torch.cuda.synchronize()
    t_gd = time.perf_counter() - t0
    first, last = float(first), float(last)
    _, _, nt, nv, _ = ctx.meshify_device(img.data_ptr(), (128, 128, 128), 50.0, n2m.MC33, True, False, False, 10)
    ctx.close()
    # FP64 host gradient of the same fixed-topology map
    from oracle.adjoint_ref import Problem
    from oracle.oracle import Oracle
    gh = Problem(Oracle(), host, 50.0, 10, center, radius).gradient(host)
    rel = float(np.linalg.norm(grad - gh) / np.linalg.norm(gh))
    fb_bytes = 4.0 * nvox + 24.0 * nv + 12.0 * nt + 12.0 * nv + 4.0 * nvox
    peak, peak_kind = peaks()
    ach = fb_bytes / (t_fb * 1e-3) / 1e9
    return {"workload": "sphere128: 128^3 f32, spheres r 12-28, iso 50, -p 1, Lewiner, 10 HC iterations",
            "fwd_ms": round(t_f, 3), "fwd_bwd_ms": round(t_fb, 3), "ratio": round(t_fb / t_f, 3),
            "grad_rel_err_vs_fp64": rel,
            "gd200_s": round(t_gd, 3), "gd_ms_per_step": round(1e3 * t_gd / gd_steps, 3),
            "gd_loss_first_last": [round(first, 2), round(last, 2)],
            "gd_loss_drop": round(1.0 - last / first, 4), "gd_optimizer": f"Adam lr {GD_LR} on the voxel values",
            "roofline": {"bound": "hbm", "bytes": fb_bytes, "achieved": round(ach, 1), "peak": peak,
                         "frac": round(ach / peak, 5), "peak_source": peak_kind,
                         "formula": "fwd (4 N_vox + 24 N_vert + 12 N_tri) + bwd (12 N_vert in, 4 N_vox out) "
                                    "per fwd+bwd wall-clock step"},
            "timing": "wall clock per step incl. host syncs (forward reads back counts)"}


def atlas_metric(n2m, torch, reps=3):
    """meshes/s on the 256^3 int16 atlas (~250 labels, -p 1 -l 1 -b 1 -s 5):
    batched all-labels path vs the per-label GPU loop, and the CPU oracle on
    a sample of labels (one core, the reference's per-label work)."""
    from nii2mesh_gb300 import synth
    lab = synth.atlas256()
    d = torch.from_numpy(lab).cuda()
    ctx = n2m.Context(torch.cuda.current_device())
    out = {"workload": "atlas256: 256^3 int16, power-law Voronoi labels, iso 0.5, -p 1 -l 1 -b 1 -s 5, Lewiner"}
    counts = {}
    for mode, name in ((n2m.ATLAS_BATCHED, "batched"), (n2m.ATLAS_LOOP, "loop")):
        ctx.atlas_device(d.data_ptr(), (256, 256, 256), mode=mode)
        ts = []
        for _ in range(reps if mode == n2m.ATLAS_BATCHED else 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            nm, ok, nv, nt, rep = ctx.atlas_device(d.data_ptr(), (256, 256, 256), mode=mode)
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        t = statistics.median(ts)
        out[f"{name}_ms"] = round(1e3 * t, 2)
        out[f"{name}_meshes_per_s"] = round(ok / t, 1)
        out["meshes"] = ok
        counts[name] = (nm, ok, nv, nt)
        if mode == n2m.ATLAS_BATCHED:
            out["batched_launches"] = rep["kernel_launches"]
            out["batched_stage_ms"] = [round(x, 3) for x in rep["ms_stage"][:5]]
            nvox = lab.size
            abytes = 2.0 * nvox + 24.0 * nv + 12.0 * nt
            peak, peak_kind = peaks()
            ach = abytes / t / 1e9
            out["roofline"] = {"bound": "hbm", "bytes": abytes, "achieved": round(ach, 1), "peak": peak,
                               "frac": round(ach / peak, 5), "peak_source": peak_kind,
                               "formula": "(2 N_vox int16 labels + sum over meshes of 24 N_vert + 12 N_tri) / "
                                          "batched wall-clock ms"}
    out["speedup_batched_vs_loop"] = round(out["batched_meshes_per_s"] / out["loop_meshes_per_s"], 2)
    out["batched_equals_loop_counts"] = counts["batched"] == counts["loop"]
    ctx.close()
    # CPU: the reference's per-label work (binarise the whole volume, meshify, 5 HC iterations), one
    # label per host core at once as its OpenMP atlas loop runs them (src/nii2mesh.c:546-574)
    import multiprocessing as mp
    ids, counts = np.unique(lab[lab > 0], return_counts=True)
    procs = host_procs(2e9)
    labels = [int(ids[i]) for i in np.argsort(counts)[np.linspace(0, len(ids) - 1, procs).astype(int)]]
    tmp = tempfile.mkdtemp(prefix="n2m_atl_", dir="/dev/shm" if os.path.isdir("/dev/shm") else None)
    path = os.path.join(tmp, "lab.npy")
    np.save(path, lab)
    mctx = mp.get_context("spawn")
    start, q = mctx.Barrier(len(labels) + 1), mctx.Queue()
    ws = [mctx.Process(target=_atlas_worker, args=(path, l, start, q), daemon=True) for l in labels]
    for w in ws:
        w.start()
    try:
        start.wait(timeout=600)
        t0 = time.perf_counter()
        for _ in labels:
            q.get(timeout=600)
        tc = time.perf_counter() - t0
    finally:
        for w in ws:
            w.join(timeout=60)
        os.remove(path)
        os.rmdir(tmp)
    out["cpu_baseline"] = {"meshes_per_s": round(len(labels) / tc, 4), "cores": len(labels), "kind": "port",
                           "sample": f"{len(labels)} labels (smallest to largest) through the full-volume per-label "
                                     f"path, one per host core ({tc:.1f} s)"}
    # the same per-label work on one core, one label after another (OMP off)
    from oracle.oracle import Oracle
    o = Oracle()
    img = lab.astype(np.float32)
    one = [labels[0], labels[len(labels) // 2], labels[-1]]
    t0 = time.perf_counter()
    for lbl in one:
        b, _ = o.binarize_label(img, lbl)
        m = o.meshify(b, 0.5, 0, True, True, True)
        if m is not None:
            o.laplacian_smoothHC(m[1], m[0], 0.1, 0.5, 5, True)
    t1 = time.perf_counter() - t0
    out["cpu_baseline_1core"] = {"meshes_per_s": round(len(one) / t1, 4), "cores": 1, "kind": "port",
                                 "sample": f"{len(one)} labels (smallest, median, largest of the sample) one after "
                                           f"another on one core ({t1:.1f} s)"}
    return out


def brain_metric(n2m, torch, reps=5):
    """The brain-sized uint8 workload (182x218x182, Otsu medium isolevel,
    -p 1 -l 1 -b 1 -s 20, Lewiner) end to end from host memory: raw uint8
    voxels through n2m_meshify_typed (cast on the device) vs the float32
    volume through n2m_meshify, and the CPU path on one core."""
    from nii2mesh_gb300 import synth
    raw = np.ascontiguousarray(synth.brain())
    vol = raw.astype(np.float32)
    ctx = n2m.Context(torch.cuda.current_device())
    iso = ctx.set_threshold(vol, 2)
    out = {"workload": "brain182: 182x218x182 uint8, Otsu medium iso, -p 1 -l 1 -b 1 -s 20, Lewiner", "iso": iso}
    for name, fn in (("u8", lambda: ctx.meshify_typed(raw, 1.0, 0.0, iso, n2m.MC33, True, True, True, 20)),
                     ("f32", lambda: ctx.meshify(vol, iso, n2m.MC33, True, True, True, 20))):
        fn()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            t, p, rep = fn()
            ts.append(time.perf_counter() - t0)
            del t, p
        out[f"e2e_{name}_ms"] = round(1e3 * statistics.median(ts), 3)
        out[f"h2d_{name}_bytes"] = int(raw.size * (1 if name == "u8" else 4))
        out["triangles"] = rep["ntri"]
    g_raw = ctx.meshify(vol, iso, n2m.MC33, True, True, True, 0)[:2]
    g_s = ctx.meshify(vol, iso, n2m.MC33, True, True, True, 20)[:2]
    ctx.close()
    from oracle.oracle import Oracle, mesh_equal, smoothed_equal
    o = Oracle()
    t0 = time.perf_counter()
    m = o.meshify(vol, iso, 0, True, True, True)
    ms = o.laplacian_smoothHC(m[1], m[0], 0.1, 0.5, 20, True)
    out["cpu_ms"] = round(1e3 * (time.perf_counter() - t0), 1)
    out["cpu_kind"] = "port"
    # parity of the same run: raw mesh bit for bit, HC positions against the oracle's FP64 HC
    ok, _, _ = mesh_equal(g_raw, m, 0.0)
    oks, d, _ = smoothed_equal(g_raw, g_s[1], m, ms, 1e-4)
    out["brain182_raw_bit_exact"] = bool(ok and np.array_equal(g_raw[0], g_s[0]))
    out["brain182_hc_max_err_vs_fp64"] = d if np.isfinite(d) else None
    return out


def threshold_metric(n2m, torch, reps=5):
    """setThreshold (Otsu on the robust range) of the brain-sized u8 volume
    (182x218x182, nii2mesh's default isolevel; medium = mode 2, dark = mode 1
    with the three-level search): device-resident, host volume through the C
    ABI, and the CPU path (one core)."""
    from nii2mesh_gb300 import synth
    vol = np.ascontiguousarray(synth.brain().astype(np.float32))
    d = torch.from_numpy(vol).cuda()
    ctx = n2m.Context(torch.cuda.current_device())
    out = {"workload": "brain182: 182x218x182 u8-valued f32 (7.2 M voxels)"}
    for mode in (2, 1):
        ctx.set_threshold_device(d.data_ptr(), vol.size, mode)
        ts, th = [], []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            iso = ctx.set_threshold_device(d.data_ptr(), vol.size, mode)
            ts.append(time.perf_counter() - t0)
            t0 = time.perf_counter()
            ctx.set_threshold(vol, mode)
            th.append(time.perf_counter() - t0)
        out[f"mode{mode}_device_ms"] = round(1e3 * statistics.median(ts), 3)
        out[f"mode{mode}_e2e_ms"] = round(1e3 * statistics.median(th), 3)
        out[f"mode{mode}_iso"] = iso
        try:
            from oracle.oracle import Reference, reference_available
            cpu = Reference(False) if reference_available() else None
            kind = "reference"
        except Exception:
            cpu = None
        if cpu is None:
            from oracle.oracle import Oracle
            cpu, kind = Oracle(), "port"
        t0 = time.perf_counter()
        ci = cpu.set_threshold(vol, mode)
        out[f"mode{mode}_cpu_ms"] = round(1e3 * (time.perf_counter() - t0), 3)
        out[f"mode{mode}_matches_cpu"] = bool(ci == iso)
        out["cpu_kind"] = kind
    ctx.close()
    return out


def variants_metric(n2m, torch, vol, reps=5):
    """The same 512^3 CT volume (device-resident) with the CLI's default clustering
    plus bubble fill (-l 1 -b 1: the clustering stage on its own) and through the
    reference's default build, the classic marching cubes of oldcubes.c (-l 0 -b 0),
    each checked against the CPU path on the same volume outside the timed region."""
    from oracle.oracle import OLDCUBES, Oracle, mesh_equal
    dev = torch.cuda.current_device()
    d = torch.from_numpy(vol).cuda()
    ctx = n2m.Context(dev)
    nx = ny = nz = vol.shape[0]
    peak, peak_kind = peaks()
    out = {}
    for name, cubes, largest, bubbles in (("ct512_l1_b1", n2m.MC33, True, True),
                                          ("ct512_oldcubes", n2m.OLDCUBES, False, False)):
        step = lambda: ctx.meshify_device(d.data_ptr(), (nx, ny, nz), ISO, cubes, True, largest, bubbles)
        for _ in range(3):
            step()
        reps_ = []
        stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(reps):
            reps_.append(step()[4])
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / reps
        r = reps_[-1]
        st = {n: round(statistics.mean(x["ms_stage"][i] for x in reps_), 4) for i, n in enumerate(STAGE_NAMES)}
        whole = 4.0 * vol.size + 24.0 * r["nvert"] + 12.0 * r["ntri"]
        gbs = whole / (ms * 1e-3) / 1e9
        out[name] = {"options": "-p 1 -l 1 -b 1 -o 0" if largest else "-p 1 -l 0 -b 0, oldcubes build",
                     "ms_per_step": round(ms, 4), "gvox_per_s": round(vol.size / (ms * 1e-3) / 1e9, 3),
                     "stage_ms": st, "triangles": r["ntri"], "vertices": r["nvert"],
                     "roofline_whole_path": {"achieved": round(gbs, 1), "frac": round(gbs / peak, 4),
                                             "peak_source": peak_kind}}
        # parity of the timed mesh against the CPU path (one host core)
        from nii2mesh_gb300.autograd import _DeviceView
        tp, pp, ntd, nvd, _ = step()
        dm = (torch.as_tensor(_DeviceView(tp, (ntd, 3), "<i4"), device=f"cuda:{dev}").cpu().numpy(),
              torch.as_tensor(_DeviceView(pp, (nvd, 3), "<f8"), device=f"cuda:{dev}").cpu().numpy())
        t0 = time.perf_counter()
        want = Oracle().meshify(vol, ISO, OLDCUBES if cubes == n2m.OLDCUBES else 0, True, largest, bubbles)
        out[name]["cpu_ms"] = round(1e3 * (time.perf_counter() - t0), 1)
        ok, dd, _ = mesh_equal(dm, want, 0.0)
        out[name]["bit_exact_vs_cpu"] = bool(ok)
        del dm, want
    ctx.close()
    return out


def writer_metric(n2m, torch, vol, reps=3):
    """save_mesh of the 512^3 CT mesh as nii2mesh writes it by default (.mz3
    gzip: quality 1 sets isGz, src/nii2mesh.c:350) and as OBJ text: the GPU
    encode of the device-resident mesh (bytes left in device memory), the whole
    n2m_save_mesh_device call (encode, readback, file write), and the CPU path
    (zlib level 6 as gzopen uses / the %g restatement, one core) on a bounded
    sample, scaled."""
    import gzip
    import tempfile
    import zlib
    from oracle import writers as W
    dev = torch.cuda.current_device()
    ctx = n2m.Context(dev)
    d = torch.from_numpy(vol).cuda()
    nz, ny, nx = vol.shape
    dt, dp, nt, nv, _ = ctx.meshify_device(d.data_ptr(), (nx, ny, nz), ISO, n2m.MC33, True, False, False)
    out = {"workload": "ct512 mesh (%d triangles, %d vertices) from the 512^3 meshify" % (nt, nv)}
    tmp = tempfile.mkdtemp(prefix="n2m_bench_")
    host = {}
    for name, fmt, gz, ext in (("mz3_gz", n2m.FMT_MZ3, True, "mz3"), ("obj", n2m.FMT_OBJ, False, "obj")):
        ctx.encode_mesh_to_device(fmt, dt, dp, nt, nv, gz)
        te, ts = [], []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _, nbytes = ctx.encode_mesh_to_device(fmt, dt, dp, nt, nv, gz)
            torch.cuda.synchronize()
            te.append(time.perf_counter() - t0)
            path = os.path.join(tmp, "mesh." + ext)
            t0 = time.perf_counter()
            ctx.save_mesh_device(path, dt, dp, nt, nv, gz)
            ts.append(time.perf_counter() - t0)
        host[name] = open(path, "rb").read()
        os.remove(path)
        out[name] = {"encode_device_ms": round(1e3 * statistics.median(te), 3),
                     "save_ms": round(1e3 * statistics.median(ts), 3), "bytes": int(nbytes)}
    raw = ctx.encode_mesh_device(n2m.FMT_MZ3, dt, dp, nt, nv, False)
    assert gzip.decompress(host["mz3_gz"]) == raw, "gzip mz3 does not decompress to the plain mz3"
    out["mz3_gz"]["ratio"] = round(len(host["mz3_gz"]) / len(raw), 4)
    # CPU: zlib level 6 on 24 MB of the body (scaled to the whole), and the ratio both get on that sample
    sample = raw[: 24 << 20]
    t0 = time.perf_counter()
    zs = zlib.compress(sample, 6)
    zt = time.perf_counter() - t0
    keep = torch.frombuffer(bytearray(sample), dtype=torch.uint8).cuda()
    ours = ctx.deflate_device(keep.data_ptr(), len(sample), n2m.DEFLATE_GZIP)
    out["mz3_gz"]["cpu"] = {"ms_scaled": round(1e3 * zt * len(raw) / len(sample), 1), "cores": 1,
                            "kind": "zlib level 6 (the reference's gzopen level)",
                            "sample": "%d MB of the mz3 body (%.2f s)" % (len(sample) >> 20, zt),
                            "zlib6_ratio_sample": round(len(zs) / len(sample), 4),
                            "gpu_ratio_sample": round(len(ours) / len(sample), 4)}
    # OBJ: the %g / %d restatement on 100k vertices + 200k triangles, scaled by lines
    tris = np.frombuffer(raw, np.int32, 3 * nt, 16).reshape(nt, 3)
    pts = np.frombuffer(raw, np.float32, 3 * nv, 16 + 12 * nt).reshape(nv, 3).astype(np.float64)
    t0 = time.perf_counter()
    W.obj(tris[:200000], pts[:100000])
    ot = time.perf_counter() - t0
    out["obj"]["cpu"] = {"ms_scaled": round(1e3 * ot * (nt + nv) / 300000, 1), "cores": 1, "kind": "port",
                         "sample": "100k vertex + 200k triangle lines (%.2f s)" % ot}
    ctx.close()
    os.rmdir(tmp)
    return out


def bench_config(world, nt, nv):
    """The workload description both arms print (the same dict for the same workload)."""
    return {"workload": WORKLOAD, "l2": "inputs larger than L2 (537 MB volume)",
            "parallelism": "replicas" if world > 1 else "single GPU", "triangles": nt, "vertices": nv}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--profile", type=int, default=0, metavar="N",
                    help="profiling driver: two meshify calls on the CT-like workload at N^3 (same generator, "
                         "structure count scaled by volume), stage times printed; no bench line")
    ap.add_argument("--largest", action="store_true", help="with --profile: keep only the largest cluster (-l 1)")
    ap.add_argument("--bubbles", action="store_true", help="with --profile: fill bubbles (-b 1)")
    ap.add_argument("--oldcubes", action="store_true", help="with --profile: the classic build's oldcubes marching cubes")
    ap.add_argument("--profile-writer", type=int, default=0, metavar="N",
                    help="profiling driver: mesh the N^3 CT-like volume, then encode it twice as .mz3 gzip and once as .obj")
    ap.add_argument("--profile-atlas", action="store_true",
                    help="profiling driver: two batched atlas calls on the 256^3 label workload; no bench line")
    a = ap.parse_args()
    warmup = max(a.warmup, 3)
    import numpy as np
    from nii2mesh_gb300 import synth

    rank, world, dist = (0, 1, None)
    if a.impl == "reference":
        if a.gpus > 1 and int(os.environ.get("RANK", "0")) != 0:
            return
        vol = synth.ct512()
        procs = host_procs()
        gv, kind, times, (nt, nv) = cpu_reference_parallel(vol, a.steps, warmup, procs)
        line = {"metric": METRIC, "value": round(gv, 6), "unit": "Gvox/s", "n_gpus": a.gpus, "steps": a.steps,
                "warmup": warmup, "ms_per_step": round(1e3 * statistics.median(times), 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
                "config": bench_config(a.gpus, nt, nv), "impl": "reference",
                "cpu_baseline": {"value": round(gv, 6), "unit": "Gvox/s", "cores": procs, "kind": kind,
                                 "sample": f"{procs} full 512^3 meshify calls per step, one per host core "
                                           f"(meshify itself is single-threaded); median of {a.steps} steps "
                                           f"after {warmup} warm-up steps"},
                "e2e": {"value": round(gv, 6), "unit": "Gvox/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch
    import nii2mesh_gb300 as n2m
    if a.profile_atlas:
        lab = synth.atlas256()
        d = torch.from_numpy(lab).cuda()
        ctx = n2m.Context(0)
        for _ in range(2):
            nm, ok, nv, nt, rep = ctx.atlas_device(d.data_ptr(), (256, 256, 256), mode=n2m.ATLAS_BATCHED)
        torch.cuda.synchronize()
        print(json.dumps({"profile_atlas": 256, "meshes": ok, "vertices": nv, "triangles": nt,
                          "stage_ms": [round(x, 4) for x in rep["ms_stage"][:5]]}))
        return
    if a.profile_writer:
        n = a.profile_writer
        pv = synth.ct512(n=n, count=max(1, int(round(300 * (n / 512) ** 3))))
        d = torch.from_numpy(pv).cuda()
        ctx = n2m.Context(0)
        dt, dp, nt, nv, _ = ctx.meshify_device(d.data_ptr(), (n, n, n), ISO, n2m.MC33, True, False, False)
        res = {}
        for fmt, gz in ((n2m.FMT_MZ3, True), (n2m.FMT_MZ3, True), (n2m.FMT_OBJ, False)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _, nb = ctx.encode_mesh_to_device(fmt, dt, dp, nt, nv, gz)
            res["mz3_gz" if gz else "obj"] = [nb, round(1e3 * (time.perf_counter() - t0), 3)]
        print(json.dumps({"profile_writer": n, "triangles": nt, "vertices": nv, "bytes_ms": res}))
        return
    if a.profile:
        n = a.profile
        pv = synth.ct512(n=n, count=max(1, int(round(300 * (n / 512) ** 3))))
        d = torch.from_numpy(pv).cuda()
        ctx = n2m.Context(0)
        for _ in range(2):
            _, _, nt, nv, rep = ctx.meshify_device(d.data_ptr(), (n, n, n), ISO, n2m.OLDCUBES if a.oldcubes else n2m.MC33,
                                                   True, a.largest, a.bubbles)
        torch.cuda.synchronize()
        print(json.dumps({"profile": n, "largest": a.largest, "bubbles": a.bubbles, "oldcubes": a.oldcubes,
                          "triangles": nt, "vertices": nv,
                          "stage_ms": dict(zip(STAGE_NAMES, [round(x, 4) for x in rep["ms_stage"][:7]]))}))
        return
    rank, world, dist = dist_setup(a.gpus)
    dev = torch.cuda.current_device()
    vol = synth.ct512()
    nx = ny = nz = 512
    nvox = vol.size
    d_vol = torch.from_numpy(vol).to(f"cuda:{dev}")
    ctx = n2m.Context(dev)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)

    def step():
        return ctx.meshify_device(d_vol.data_ptr(), (nx, ny, nz), ISO, n2m.MC33, True, False, False)

    for _ in range(warmup):
        step()
    reps = []
    clocks = Clocks(dev)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(a.steps):
        reps.append(step()[4])
    ev1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    if dist:
        dist.barrier()
    ms = slowest_rank_ms(ev0.elapsed_time(ev1) / a.steps, dist, f"cuda:{dev}")
    value = job_value(nvox, world, ms)
    nt, nv = reps[-1]["ntri"], reps[-1]["nvert"]
    launches = sum(r["kernel_launches"] for r in reps)
    stage_ms = [statistics.mean(r["ms_stage"][i] for r in reps) for i in range(7)]

    # roofline of the dominant stage (algorithmic bytes / CUDA-event duration), every stage's
    # figure beside it, and the whole path's: 4 B/voxel read once + 24 B/vertex + 12 B/triangle
    # written once, over the whole step
    lo, hi = reps[-1]["lo"], reps[-1]["hi"]
    ngrid = (hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1)
    nv_raw, nt_raw = reps[-1]["nvert_raw"], reps[-1]["ntri_raw"]
    algo = {"smooth": 8.0 * nvox, "count": 4.0 * ngrid, "emit": 24.0 * nv_raw + 12.0 * nt_raw,
            "weld": 24.0 * nv_raw + 24.0 * nv + 24.0 * nt_raw, "degenerate": 24.0 * nt_raw}
    peak, peak_kind = peaks()
    stages = {}
    for i, nm in enumerate(STAGE_NAMES):
        if nm not in algo or stage_ms[i] <= 0:
            continue
        ach = algo[nm] / (stage_ms[i] * 1e-3) / 1e9
        st = {"ms": round(stage_ms[i], 4), "algorithmic_bytes": algo[nm], "achieved_gbs": round(ach, 1),
              "frac": round(ach / peak, 4)}
        if nm in NCU_TRAFFIC:
            st["dram_bytes"] = NCU_TRAFFIC[nm]
            st["dram_over_algorithmic"] = round(NCU_TRAFFIC[nm] / algo[nm], 2)
        stages[nm] = st
    whole = 4.0 * nvox + 24.0 * nv + 12.0 * nt
    whole_gbs = whole / (ms * 1e-3) / 1e9
    # the dominant kernel: pass A of the pre-smooth (k_od_approx), 4 B read + 4 B written + 1/8 B of
    # sign bitmap per voxel, over its own CUDA-event time on the library's stream
    pa_ms = statistics.mean(r.get("ms_smooth_pass_a", 0.0) for r in reps)
    pa_bytes = 8.125 * nvox
    pa_gbs = pa_bytes / (pa_ms * 1e-3) / 1e9 if pa_ms > 0 else None
    roof = {"bound": "hbm", "kernel": "k_od_approx (pre-smooth pass A)", "achieved": round(pa_gbs, 1) if pa_gbs else None,
            "peak": peak, "unit": "GB/s", "frac": round(pa_gbs / peak, 4) if pa_gbs else None, "peak_source": peak_kind,
            "kernel_ms": round(pa_ms, 4), "algorithmic_bytes": pa_bytes, "traffic": PASS_A_TRAFFIC,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_od_approx launch at 384^3, "
                              "scaled by the voxel count",
            "limited_by": "FP32 instruction issue (74 % issue active); memory 1.9-2.4 TB/s",
            "whole_path": {"bytes": whole, "achieved": round(whole_gbs, 1), "frac": round(whole_gbs / peak, 4),
                           "formula": "(4 N_vox + 24 N_vert + 12 N_tri) / ms_per_step / peak",
                           "dram_bytes": round(sum(NCU_TRAFFIC.values())),
                           "dram_over_algorithmic": round(sum(NCU_TRAFFIC.values()) / whole, 2)},
            "stages": stages, "stage_bounds": STAGE_BOUND}

    # e2e through the C ABI with host buffers: the volume from pinned memory, the mesh copied back into
    # pinned arrays the caller allocates once and reuses (n2m_meshify_into); the malloc-returning
    # n2m_meshify (the reference's ownership contract) is timed beside it
    pinned = torch.from_numpy(vol).pin_memory().numpy()
    tris, pts, _ = ctx.meshify(pinned, ISO, n2m.MC33, True, False, False)
    tbuf = torch.empty((len(tris) + 4096, 3), dtype=torch.int32, pin_memory=True).numpy()
    pbuf = torch.empty((len(pts) + 4096, 3), dtype=torch.float64, pin_memory=True).numpy()
    for _ in range(2):
        ctx.meshify_into(pinned, tbuf, pbuf, ISO, n2m.MC33, True, False, False)
    e2e_t, e2e_malloc = [], []
    for _ in range(a.steps):
        t0 = time.perf_counter()
        nt_e, nv_e, _ = ctx.meshify_into(pinned, tbuf, pbuf, ISO, n2m.MC33, True, False, False)
        e2e_t.append(time.perf_counter() - t0)
    assert (nt_e, nv_e) == (len(tris), len(pts))
    for _ in range(a.steps):
        t0 = time.perf_counter()
        tris, pts, _ = ctx.meshify(pinned, ISO, n2m.MC33, True, False, False)
        e2e_malloc.append(time.perf_counter() - t0)
    e2e_ms = slowest_rank_ms(statistics.median(e2e_t) * 1e3, dist, f"cuda:{dev}")
    e2e = {"value": round(world * nvox / (e2e_ms * 1e-3) / 1e9, 4), "unit": "Gvox/s",
           "h2d_bytes_per_step": 4 * nvox, "d2h_bytes_per_step": 24 * nv_e + 12 * nt_e,
           "ms_per_step": round(e2e_ms, 3), "call": "n2m_meshify_into (pinned volume, reused pinned mesh arrays)",
           "malloc_call_ms": round(statistics.median(e2e_malloc) * 1e3, 3)}

    if rank != 0:
        return
    cpu, parity = None, {}
    if world == 1:
        from oracle.oracle import mesh_equal
        gv, kind, times, cmesh = cpu_reference(vol, 1, 0)
        cpu = {"value": round(gv, 6), "unit": "Gvox/s", "cores": 1, "kind": kind,
               "sample": f"one full 512^3 meshify ({times[0]:.1f} s)"}
        # the meshes the timed calls produce (the device-resident step and the last host-memory
        # call) against the CPU path's, outside the timed region
        from nii2mesh_gb300.autograd import _DeviceView
        tp, pp, ntd, nvd, _ = step()
        dmesh = (torch.as_tensor(_DeviceView(tp, (ntd, 3), "<i4"), device=f"cuda:{dev}").cpu().numpy(),
                 torch.as_tensor(_DeviceView(pp, (nvd, 3), "<f8"), device=f"cuda:{dev}").cpu().numpy())
        okd, dd, msgd = mesh_equal(dmesh, cmesh, 0.0)
        ok, d, msg = mesh_equal((tris, pts), cmesh, 0.0)
        parity = {"ct512_bit_exact": bool(ok and okd), "ct512_max_dpos": max(d, dd) if np.isfinite(max(d, dd)) else None,
                  "ct512_detail": f"device step: {msgd}; host call: {msg}", "ct512_against": kind,
                  "rule": "identical counts and canonical connectivity; positions within 0 (raw) / 1e-4 (HC) voxels"}
        del dmesh
        del cmesh
    adj = adjoint_metric(n2m, torch) if world == 1 else None
    atl = atlas_metric(n2m, torch) if world == 1 else None
    thr = threshold_metric(n2m, torch) if world == 1 else None
    brn = brain_metric(n2m, torch) if world == 1 else None
    wrt = writer_metric(n2m, torch, vol) if world == 1 else None
    var = variants_metric(n2m, torch, vol) if world == 1 else None
    line = {"metric": METRIC, "value": round(value, 4), "unit": "Gvox/s", "n_gpus": world, "steps": a.steps,
            "warmup": warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
            "config": bench_config(world, nt, nv),
            "stage_ms": {n: round(v, 4) for n, v in zip(STAGE_NAMES, stage_ms)},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": ck,
            "parity": parity, "adjoint": adj, "atlas": atl, "threshold": thr, "brain": brn, "writer": wrt,
            "variants": var}
    if var:
        parity.update({f"{k}_bit_exact": v.pop("bit_exact_vs_cpu") for k, v in var.items()})
    if brn:
        parity.update({k: brn.pop(k) for k in ("brain182_raw_bit_exact", "brain182_hc_max_err_vs_fp64")})
    if adj:
        parity["adjoint128_grad_rel_err_vs_fp64"] = adj.pop("grad_rel_err_vs_fp64")
    if atl:
        parity["atlas256_batched_equals_loop_counts"] = atl.pop("batched_equals_loop_counts")
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
