"""Benchmark of the 3D VTI FD hot path on the 400^3 workload.

Workload (one bench step = one full shot): 400x400x400 grid + 40-cell
sponge (480^3 padded), dx=dy=dz=10 m, dt=0.8 ms, 2500 time steps, FP32,
15 Hz Ricker at the surface centre, 200x200 receivers (every 2nd surface
node).  Model: seeded smooth Gaussian random field (correlation length 40
cells) plus 3 dipping interfaces, vp 1500-4500 m/s, eps = 0.3*(vp-1500)/3000,
del = 0.15*(vp-1500)/3000.  Synthetic, generated on the fly.

Metric: grid-point updates per second, counting the points the step
updates ((nn-8)^3 per time step).  `value` runs shots with the model and
wavefields resident in HBM; `e2e` goes through the C ABI with host buffers
(model upload and record download inside the timed region).  The working
set (~10 GB) is far larger than L2, so no flush is needed between steps.

--impl reference times the CPU restatement of the same step (the reference
has no CPU code for 3D VTI) with all host threads on a bounded sample.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX = NY = NZ = 400
NPD = 40
NT = 2500
DT = 0.0008
DX = 10.0
FAVG = 15.0
CFG = {"workload": "3D VTI FD shot 400^3 (+40 sponge), 2500 steps, dt=0.8 ms, 10 m, 15 Hz Ricker, "
                   "200x200 receivers", "grid": [NX, NY, NZ], "sponge": NPD, "nt": NT,
       "stress_form": "fast (unsplit interior)", "l2": "inputs larger than L2 (no flush)"}


def updates_per_step():
    return (NX + 2 * NPD - 8) * (NY + 2 * NPD - 8) * (NZ + 2 * NPD - 8)


def algorithmic_bytes_per_step():
    """52 B per interior update (read u,v,w,P,Q + 3 coefficients, write
    u,v,w,P,Q) and 84 B per sponge update (read/write u,v,w and 6 split
    stresses, read 3 coefficients)."""
    interior = NX * NY * NZ
    sponge = updates_per_step() - interior
    return interior * 52 + sponge * 84


def make_model(seed=2, device="cuda"):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    noise = torch.randn((NY, NX, NZ), generator=g, dtype=torch.float32).to(device)
    L = 40.0
    sig = L / 2.0
    fy = torch.fft.fftfreq(NY, device=device)[:, None, None]
    fx = torch.fft.fftfreq(NX, device=device)[None, :, None]
    fz = torch.fft.rfftfreq(NZ, device=device)[None, None, :]
    filt = torch.exp(-2.0 * (torch.pi ** 2) * sig ** 2 * (fx ** 2 + fy ** 2 + fz ** 2))
    G = torch.fft.irfftn(torch.fft.rfftn(noise) * filt, s=(NY, NX, NZ))
    G = (G - G.min()) / (G.max() - G.min())
    vp = 1500.0 + 2100.0 * G
    iy = torch.arange(NY, device=device, dtype=torch.float32)[:, None, None]
    ix = torch.arange(NX, device=device, dtype=torch.float32)[None, :, None]
    iz = torch.arange(NZ, device=device, dtype=torch.float32)[None, None, :]
    for z0, ax, ay in ((110.0, 0.10, 0.05), (210.0, -0.08, 0.12), (300.0, 0.05, -0.10)):
        vp = vp + 300.0 * (iz > z0 + ax * (ix - NX / 2) + ay * (iy - NY / 2)).float()
    eps = 0.3 * (vp - 1500.0) / 3000.0
    dl = 0.15 * (vp - 1500.0) / 3000.0
    return vp.float().contiguous(), eps.float().contiguous(), dl.float().contiguous()


def plan_kwargs():
    return dict(nx=NX, ny=NY, nz=NZ, npd=NPD, nt=NT, dx=DX, dy=DX, dz=DX, dt=DT, favg=FAVG, pfac=10.0,
                fsx=NX // 2, fsy=NY // 2, fsz=1, mode="fast", rec_iz=NPD, rx0=0, drx=2, nrx=200, ry0=0, dry=2,
                nry=200)


class Clocks:
    """nvidia-smi samples during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
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
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                mx = max(mx, float(p[1]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if p[3 + k].lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_sample(steps):
    """The oracle's OpenMP step on the full grid for `steps` time steps:
    returns updates/s and the threads used."""
    import numpy as np

    from oracle import orc
    vp, eps, dl = (a.cpu().numpy() for a in make_model(device="cpu"))
    t0 = time.perf_counter()
    orc.fd3d(vp, eps, dl, npd=NPD, nt=steps, dx=DX, dy=DX, dz=DX, dt=np.float32(DT), favg=FAVG, pfac=10.0,
             fsx=NX // 2, fsy=NY // 2, fsz=1, mode=1, drx=2, nrx=200, dry=2, nry=200)
    dt = time.perf_counter() - t0
    return updates_per_step() * steps / dt, dt


def run_reference(args, rank):
    if rank != 0:
        return
    from oracle import orc
    orc.build(with_ref=False)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    sample_steps = 4
    for _ in range(args.warmup):
        cpu_sample(sample_steps)
    vals, secs = [], []
    for _ in range(args.steps):
        v, s = cpu_sample(sample_steps)
        vals.append(v)
        secs.append(s)
    value = sum(vals) / len(vals) / 1e9
    line = {"impl": "reference", "metric": "grid-pt updates/s", "value": value, "unit": "Gpt/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * statistics.mean(secs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": CFG,
            "cpu_baseline": {"value": value, "unit": "Gpt/s", "cores": cores, "kind": "port",
                             "sample": "%d time steps of the full 480^3 grid per bench step (the reference has no "
                                       "3D CPU code; this is the oracle's OpenMP restatement, fast form)" % sample_steps},
            "e2e": {"value": value, "unit": "Gpt/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world):
    import numpy as np
    import torch

    import geophysics_gb300 as geo
    from geophysics_gb300 import build as B
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    B.build()
    vp, eps, dl = make_model(device="cuda")
    plan = geo.FD3DPlan(**plan_kwargs())
    plan.set_model(vp, eps, dl)
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        plan.run_shot(0, device="cuda")
    barrier()
    l0 = geo.launch_count()
    with Clocks(dev) as clk:
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        ev0.record(stream)
        for _ in range(args.steps):
            plan.run_shot(0, device="cuda")
        ev1.record(stream)
        barrier()
    launches = geo.launch_count() - l0
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    value = world * updates_per_step() * NT / (ms_step / 1000) / 1e9

    # roofline: bare time steps of the stencil on the launching stream
    nsteps = 50
    step_ms = plan.time_steps(nsteps, stream=torch.cuda.current_stream().cuda_stream) / nsteps
    peak, peak_kind = measured_peak()
    achieved = algorithmic_bytes_per_step() / (step_ms / 1000) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "fd3d_fused_400cube_traffic.md")
    if os.path.exists(tf):
        for line in open(tf):
            if line.startswith("bytes_per_step:"):
                traffic = int(line.split(":")[1])

    # end to end through the C ABI with host buffers
    hv, he, hd = (a.cpu().numpy() for a in (vp, eps, dl))
    del vp, eps, dl
    plan.set_model(hv, he, hd)
    plan.run_shot(0)
    barrier()
    e2e_steps = max(1, args.steps)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        plan.set_model(hv, he, hd)
        rec = plan.run_shot(0)
    barrier()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": world * updates_per_step() * NT / e2e_s / 1e9, "unit": "Gpt/s",
           "h2d_bytes_per_step": int(hv.nbytes + he.nbytes + hd.nbytes), "d2h_bytes_per_step": int(rec.nbytes)}
    plan.close()
    if rank != 0:
        return
    cpu = None
    if world == 1 and not args.no_cpu:
        cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
        cval, csec = cpu_sample(4)
        cpu = {"value": cval / 1e9, "unit": "Gpt/s", "cores": cores, "kind": "port",
               "sample": "4 time steps of the full 480^3 grid (%.1f s); oracle OpenMP restatement, fast form" % csec}
    line = {"metric": "grid-pt updates/s", "value": value, "unit": "Gpt/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": dict(CFG, parallelism="replicas"),
            "e2e": e2e, "gpu_launches": launches, "clocks": clk.summary(),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "peak_kind": peak_kind, "unit_of_work": "one time step (%d updates, "
                         "%.3f GB algorithmic)" % (updates_per_step(), algorithmic_bytes_per_step() / 1e9),
                         "step_ms": step_ms},
            "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)


def run_profile_case(args):
    """Small case for ncu captures: 192^3 + 40 sponge (272^3 padded, each
    field 80 MB, the working set well above L2), a 20-step shot."""
    import torch

    import geophysics_gb300 as geo
    global NX, NY, NZ
    NX = NY = NZ = 192
    vp, eps, dl = make_model(device="cuda")
    kw = plan_kwargs()
    kw.update(nt=20, nrx=96, nry=96)
    plan = geo.FD3DPlan(**kw)
    plan.set_model(vp, eps, dl)
    for _ in range(args.steps):
        plan.run_shot(0, device="cuda")
    torch.cuda.synchronize()
    plan.close()
    print(json.dumps({"case": "profile-small", "grid": 192, "nt": 20, "shots": args.steps}))


def run_traffic_case(args):
    """The full 400^3 grid with a handful of bare time steps, for a one-pass
    ncu capture of the stencil's DRAM bytes per launch."""
    import torch

    import geophysics_gb300 as geo
    vp, eps, dl = make_model(device="cuda")
    plan = geo.FD3DPlan(**plan_kwargs())
    plan.set_model(vp, eps, dl)
    plan.time_steps(max(1, args.steps))
    torch.cuda.synchronize()
    plan.close()
    print(json.dumps({"case": "traffic", "grid": NX, "steps": args.steps}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--case", default="full", choices=["full", "small", "traffic"],
                    help="small / traffic: ncu profiling cases (not a bench line)")
    args = ap.parse_args()
    if args.case == "small":
        run_profile_case(args)
        return
    if args.case == "traffic":
        run_traffic_case(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.init_process_group("nccl")
    if args.impl == "reference":
        run_reference(args, rank)
    else:
        run_ours(args, rank, world)
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
