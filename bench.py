"""Benchmark of the 3D VTI FD hot path on the 400^3 workload.

Workload (one bench step = one full shot): 400x400x400 grid + 40-cell
sponge (480^3 padded), dx=dy=dz=10 m, dt=0.8 ms, 2500 time steps, FP32,
15 Hz Ricker at the surface centre, 200x200 receivers (every 2nd surface
node).  Model: seeded smooth Gaussian random field (correlation length 40
cells) plus 3 dipping interfaces, vp 1500-4500 m/s, eps = 0.3*(vp-1500)/3000,
del = 0.15*(vp-1500)/3000.  Synthetic, generated on the fly.

Metric: grid-point updates per second, counting the points the step
updates ((nn-8)^3 per time step).  `value` runs shots with the model and
wavefields resident in HBM; `e2e` goes through the C ABI with pinned host
buffers (model upload and record download inside the timed region).  The working
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


# DRAM bytes (read + write) of one launch of the fused step at 400^3 + 40,
# from ncu on the 200^3 + 20 case (same sponge fraction, 240^3 padded, a
# few GB on the device) scaled by the updated points (472/232)^3; command and
# figures in profiles/fd3d_fused_200cube_traffic.md.
TRAFFIC_BYTES_PER_STEP = 8665488602


def updates_per_step():
    return (NX + 2 * NPD - 8) * (NY + 2 * NPD - 8) * (NZ + 2 * NPD - 8)


def algorithmic_bytes_per_step():
    """52 B per interior update (read u,v,w,P,Q + 3 coefficients, write
    u,v,w,P,Q) and 84 B per sponge update (read/write u,v,w and 6 split
    stresses, read 3 coefficients)."""
    interior = NX * NY * NZ
    sponge = updates_per_step() - interior
    return interior * 52 + sponge * 84


def make_model(seed=2, device="cuda", shape=None, corr=40.0):
    """Seeded Gaussian random field (correlation `corr` cells) plus 3 dipping
    interfaces; (ny, nx, nz) tensors vp, eps, del."""
    import torch
    ny, nx, nz = shape or (NY, NX, NZ)
    g = torch.Generator(device="cpu").manual_seed(seed)
    noise = torch.randn((ny, nx, nz), generator=g, dtype=torch.float32).to(device)
    sig = corr / 2.0
    fy = torch.fft.fftfreq(ny, device=device)[:, None, None]
    fx = torch.fft.fftfreq(nx, device=device)[None, :, None]
    fz = torch.fft.rfftfreq(nz, device=device)[None, None, :]
    filt = torch.exp(-2.0 * (torch.pi ** 2) * sig ** 2 * (fx ** 2 + fy ** 2 + fz ** 2))
    G = torch.fft.irfftn(torch.fft.rfftn(noise) * filt, s=(ny, nx, nz))
    G = (G - G.min()) / (G.max() - G.min())
    vp = 1500.0 + 2100.0 * G
    iy = torch.arange(ny, device=device, dtype=torch.float32)[:, None, None]
    ix = torch.arange(nx, device=device, dtype=torch.float32)[None, :, None]
    iz = torch.arange(nz, device=device, dtype=torch.float32)[None, None, :]
    for fz0, ax, ay in ((0.275, 0.10, 0.05), (0.525, -0.08, 0.12), (0.75, 0.05, -0.10)):
        vp = vp + 300.0 * (iz > fz0 * nz + ax * (ix - nx / 2) + ay * (iy - ny / 2)).float()
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
    traffic = TRAFFIC_BYTES_PER_STEP

    # end to end through the C ABI with host buffers: the model from pinned
    # host memory, the record read back into pinned host memory
    pinned = [torch.empty(a.shape, dtype=torch.float32, pin_memory=True) for a in (vp, eps, dl)]
    for h, a in zip(pinned, (vp, eps, dl)):
        h.copy_(a)
    hv, he, hd = (h.numpy() for h in pinned)
    del vp, eps, dl
    D = plan.desc
    rec_pin = torch.empty((D.nry, D.nrx, D.nt), dtype=torch.float32, pin_memory=True)
    rec = rec_pin.numpy()
    plan.set_model(hv, he, hd)
    plan.run_shot(0, out=rec)
    barrier()
    e2e_steps = max(1, args.steps)
    with Clocks(dev) as clk_e2e:
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            plan.set_model(hv, he, hd)
            plan.run_shot(0, out=rec)
        barrier()
        e2e_s = (time.perf_counter() - t0) / e2e_steps
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = {"value": world * updates_per_step() * NT / e2e_s / 1e9, "unit": "Gpt/s",
           "h2d_bytes_per_step": int(hv.nbytes + he.nbytes + hd.nbytes), "d2h_bytes_per_step": int(rec.nbytes),
           "clocks": clk_e2e.summary()}
    plan.close()
    # the exact stress form (the reference's FP32 arithmetic, bit-identical to
    # the oracle) on the same grid, bare steps, for callers that need it
    pex = geo.FD3DPlan(**dict(plan_kwargs(), mode="exact"))
    pex.set_model(hv, he, hd)
    pex.time_steps(5, stream=torch.cuda.current_stream().cuda_stream)
    exact_ms = pex.time_steps(nsteps, stream=torch.cuda.current_stream().cuda_stream) / nsteps
    pex.close()
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
            "cpu_baseline": cpu,
            "exact_form": {"step_ms": exact_ms, "value": updates_per_step() / (exact_ms / 1000) / 1e9,
                           "unit": "Gpt/s",
                           # the same algorithmic bytes as the headline (52 B interior,
                           # 84 B sponge): what the step must move, not what this form moves
                           "roofline_frac": algorithmic_bytes_per_step() / (exact_ms / 1000) / 1e9 / peak,
                           "note": "bare steps of the reference-arithmetic form, bit-identical to the reference "
                           "program built without FMA contraction; it keeps the split stresses everywhere "
                           "(84 B moved per update); the headline fast form's record is 1.08e-5 rel-L2 from it "
                           "after 2500 steps, and the reference program's own default and no-FMA builds are "
                           "2.25e-5 apart on this shot"}}
    print(json.dumps(line), flush=True)


def run_profile_case(args):
    """Small case for ncu captures: by default 192^3 + 40 sponge (272^3
    padded, each field 80 MB, the working set well above L2), a 20-step
    shot; --grid / --sponge change the cube (200 and 20 give the headline
    case's sponge fraction)."""
    import torch

    import geophysics_gb300 as geo
    global NX, NY, NZ
    NX = NY = NZ = args.grid = args.grid or 192
    vp, eps, dl = make_model(device="cuda")
    kw = plan_kwargs()
    kw.update(nt=20, nrx=args.grid // 2, nry=args.grid // 2, npd=args.sponge, rec_iz=args.sponge)
    plan = geo.FD3DPlan(**kw)
    plan.set_model(vp, eps, dl)
    for _ in range(args.steps):
        plan.run_shot(0, device="cuda")
    torch.cuda.synchronize()
    plan.close()
    print(json.dumps({"case": "profile-small", "grid": args.grid, "sponge": args.sponge, "nt": 20, "shots": args.steps}))


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


def smooth_field(shape, corr, seed, device="cuda"):
    """Seeded Gaussian random field (FFT-filtered white noise, correlation
    `corr` cells) scaled to [0, 1]."""
    import torch
    ny, nx, nz = shape
    g = torch.Generator(device="cpu").manual_seed(seed)
    noise = torch.randn(shape, generator=g, dtype=torch.float32).to(device)
    sig = corr / 2.0
    fy = torch.fft.fftfreq(ny, device=device)[:, None, None]
    fx = torch.fft.fftfreq(nx, device=device)[None, :, None]
    fz = torch.fft.rfftfreq(nz, device=device)[None, None, :]
    filt = torch.exp(-2.0 * (torch.pi ** 2) * sig ** 2 * (fx ** 2 + fy ** 2 + fz ** 2))
    f = torch.fft.irfftn(torch.fft.rfftn(noise) * filt, s=shape)
    return ((f - f.min()) / (f.max() - f.min())).float().contiguous()


def tti_model(shape, seed=5, device="cuda"):
    """3D TTI medium: vp as make_model (random field + dipping interfaces),
    eps = 0.3 r and del = -0.05 + 0.2 r with r = (vp - 1500) / 3000 (so
    del < eps everywhere: the pseudo-acoustic TTI scheme is unstable where
    del > eps), tilt 0-45 deg and azimuth 0-360 deg as seeded smooth fields
    (correlation 60 cells)."""
    vp, _, _ = make_model(seed=seed, device=device, shape=shape)
    r = ((vp - 1500.0) / 3000.0).clamp(0, 1)
    eps = (0.3 * r).float().contiguous()
    dl = (-0.05 + 0.2 * r).float().contiguous()
    theta = (45.0 * smooth_field(shape, 60.0, seed + 1000, device)).contiguous()
    phi = (360.0 * smooth_field(shape, 60.0, seed + 2000, device)).contiguous()
    return vp, eps, dl, theta, phi


def train_codec(geo, iters, models=32, n=96, seed=1, tti=False):
    """The codec trained on snapshots the solver generates: `models` seeded
    random-field media of n^3 (correlation 8-40 cells, random surface
    source), P every 12 steps of a 560-step shot (SV taper on); with `tti`
    the media are 3D TTI (tti_model) at n^3."""
    import numpy as np
    import torch
    codec = geo.Codec(seed=seed)
    codec.reserve(150000)
    rng = np.random.default_rng(seed)
    kw = dict(npd=16, nt=560, dx=DX, dy=DX, dz=DX, dt=DT, favg=FAVG, fsz=1, mode="fast", sv=1)
    t0 = time.perf_counter()
    for s in range(models):
        if tti:
            v, e, d, th, ph = tti_model((n, n, n), seed=100 + s)
        else:
            v, e, d = make_model(seed=100 + s, device="cuda", shape=(n, n, n), corr=float(rng.uniform(8, 40)))
        plan = geo.FD3DPlan(nx=n, ny=n, nz=n, fsx=int(rng.integers(16, n - 16)), fsy=int(rng.integers(16, n - 16)),
                            **kw)
        plan.set_model(v, e, d)
        if tti:
            plan.set_tilt(th, ph)
        codec.add_shot(plan, 0, snap_every=12, t_first=8)
        plan.close()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    loss = codec.train(iters, batch=256, lr=1e-3)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return codec, {"models": models, "grid": n, "blocks": codec.num_blocks(), "iters": iters,
                   "collect_s": round(t1 - t0, 2), "train_s": round(t2 - t1, 2), "final_loss": float(loss[-50:].mean())}


def run_rtm_learned_case(args):
    """3D VTI RTM, one shot, 512x512x384 at 10 m (+40 sponge), dt 0.8 ms,
    15 Hz: the plain recomputes (the program's boundary re-propagation and
    the exact checkpoint recompute) against snapshots every 4 steps through
    the learned codec (shots/hour), and the codec's image error over the
    whole run against the exact checkpoint recompute's image (bit for bit
    the image of stored fp32 snapshots, which would need 302 GB here)."""
    import numpy as np
    import torch

    import geophysics_gb300 as geo
    from geophysics_gb300 import build as B
    B.build()
    nx, ny, nz = 512, 512, 384
    vp, eps, dl = make_model(seed=4, device="cuda", shape=(ny, nx, nz))
    rk = dict(npd=NPD, dx=DX, dy=DX, dz=DX, dt=DT, favg=FAVG, fsx=nx // 2, fsy=ny // 2, fsz=1, mute_tt=70,
              laplace=True, mode="fast", sv=1)
    codec, tinfo = train_codec(geo, args.train_iters)

    def timed(**kw):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = geo.rtm3d(vp, eps, dl, **rk, **kw)
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    res = {}
    bnd, res["boundary"] = timed(nt=args.nt, method="boundary")
    ref, res["checkpoint"] = timed(nt=args.nt, method="checkpoint", snap_every=4)
    codec.set_escape(0.02, 0.0)
    l16, res["learned16"] = timed(nt=args.nt, method="learned", snap_every=4, codec=codec)
    codec.set_escape(0.02, args.escape)
    b0, e0 = codec.stats()
    les, res["learned_esc"] = timed(nt=args.nt, method="learned", snap_every=4, codec=codec)
    b1, e1 = codec.stats()

    def rel(a, b):
        a, b = a[0].double(), b[0].double()
        return float((a - b).norm() / b.norm())

    esc_frac = (e1 - e0) / max(1, b1 - b0)

    def per_block(f):   # bytes per 16^3 block: code, scale, escape slot map, residuals
        return 1024 + 4 + 4 + f * 8192
    line = {"case": "rtm-learned", "metric": "3D RTM shots/hr, learned snapshot codec vs boundary-saving recompute",
            "grid": [nx, ny, nz], "sponge": NPD, "nt": args.nt, "snap_every": 4,
            "shots_per_hr": {k: 3600.0 / v for k, v in res.items()}, "seconds": res,
            "speedup_vs_boundary": {"learned16": res["boundary"] / res["learned16"],
                                    "learned_esc": res["boundary"] / res["learned_esc"]},
            "speedup_vs_checkpoint": {"learned16": res["checkpoint"] / res["learned16"],
                                      "learned_esc": res["checkpoint"] / res["learned_esc"]},
            "image_rel_l2_vs_plain": {"learned16": rel(l16, ref), "learned_esc": rel(les, ref),
                                      "boundary": rel(bnd, ref), "steps": args.nt,
                                      "plain": "checkpoint recompute (= stored fp32 snapshots bit for bit)",
                                      "image": "Laplacian-filtered, illumination-divided"},
            "compression": {"learned16": 16384 / per_block(0.0),
                            "learned_esc": 16384 / per_block(esc_frac), "escaped_block_frac": esc_frac,
                            "escape_budget": args.escape},
            "training": tinfo, "dtype": "f32 propagation, bf16 codec", "data": "synthetic"}
    print(json.dumps(line), flush=True)


TTI_SHAPE, TTI_DX, TTI_DT, TTI_FAVG, TTI_NT = (600, 600, 400), 12.5, 0.0008, 12.0, 3500
TTI_BYTES_PER_PT = 104   # velocity kernel 12 floats (P,Q,u,v,w,4 trig in; u,v,w out), stress 14


def run_prog2d_case(args):
    """The 2D GPU programs at their own sizes, device buffers: the 2D TTI
    forward shot at the TTI program's 600x300 (5 m, npml 50, 801 steps,
    40 Hz, dt 0.5 ms, source (200, 140)) and one shot of each 2D GPU RTM
    program on the TTI RTM program's 1700x601 (5 m, npml 50, 2000 of its
    9001 steps, 20 Hz); seeded layered VTI media, tilt 25 +- 20 deg as a
    smooth field.  Median wall time per call."""
    import numpy as np
    import torch

    import geophysics_gb300 as geo
    from geophysics_gb300 import build as B
    from geophysics_gb300 import media
    B.build()

    def tilt(nx, nz):
        x, z = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
        return (25 + 20 * np.sin(x / 40.0) * np.cos(z / 30.0)).astype(np.float32)

    def timed(fn, reps):
        for _ in range(max(args.warmup, 1)):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return 1000 * statistics.median(ts)

    v, e, d = media.layered_vti(600, 300, seed=1)
    t = [torch.from_numpy(a).cuda() for a in (v, e, d, tilt(600, 300))]
    kw = dict(npd=50, nt=801, dx=5.0, dz=5.0, dt=5e-4, favg=40.0, fs=200, zs=140)
    res = {"tti2d_shot_600x300_801_ms": timed(lambda: geo.tti2d_shot(*t, **kw), max(args.steps, 5))}
    v, e, d = media.layered_vti(1700, 601, seed=2)
    t = [torch.from_numpy(a).cuda() for a in (v, e, d, tilt(1700, 601))]
    kr = dict(npml=50, nt=2000, dx=5.0, dz=5.0, dt=5e-4, favg=20.0, ns=1, fs=850, zs=1)
    res["rtm2d_tti_1700x601_2000_ms"] = timed(lambda: geo.rtm2d_tti(*t, **kr), max(args.steps, 3))
    res["rtm2d_gpu_1700x601_2000_ms"] = timed(lambda: geo.rtm2d_gpu(*t[:3], **kr), max(args.steps, 3))
    print(json.dumps({"case": "prog2d", "unit": "ms", **res, "dtype": "f32", "data": "synthetic"}), flush=True)


def run_codec_case(args):
    """The learned snapshot codec alone: encode + decode of one 512x512x384
    snapshot (24 576 blocks of 16^3, the 3D RTM comparison's grid) as
    Codec.roundtrip runs it (E1 gather, six tcgen05 GEMM levels, D1
    scatter).  Input: seeded Gaussian noise smoothed by a 5^3 box filter;
    untrained weights (the codec's speed does not depend on them).  Each
    call allocates its code buffers, so the time includes those
    allocations."""
    import torch

    import geophysics_gb300 as geo
    from geophysics_gb300 import build as B
    B.build()
    g = torch.Generator(device="cuda").manual_seed(3)
    vol = torch.randn((512, 512, 384), device="cuda", generator=g)
    vol = torch.nn.functional.avg_pool3d(vol[None, None], 5, stride=1, padding=2)[0, 0].contiguous()
    cd = geo.Codec(seed=1)
    for _ in range(max(args.warmup, 3)):
        cd.roundtrip(vol)
    torch.cuda.synchronize()
    times = []
    for _ in range(max(args.steps, 5)):
        t0 = time.perf_counter()
        cd.roundtrip(vol)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    print(json.dumps({"case": "codec", "metric": "codec encode+decode ms per snapshot",
                      "value": 1000 * statistics.median(times), "unit": "ms", "min_ms": 1000 * min(times),
                      "blocks": 24576, "grid": [512, 512, 384], "dtype": "bf16 codec", "data": "synthetic"}),
          flush=True)
    cd.close()


def run_tti_case(args):
    """Bare 3D TTI time steps on the 600x600x400 (+40 sponge) medium at
    12.5 m, dt 0.8 ms (tti_model): updates/s and the two kernels' roofline
    (104 algorithmic bytes per updated point against the measured copy
    peak).  cpu: the oracle's FP32 TTI restatement (OpenMP, all host
    cores) on a 120^3 + 20 sample, 10 steps."""
    import numpy as np
    import torch

    import geophysics_gb300 as geo
    from geophysics_gb300 import build as B
    B.build()
    shape = (args.grid,) * 3 if args.grid else TTI_SHAPE
    ny, nx, nz = shape
    v, e, d, th, ph = tti_model(shape)
    plan = geo.FD3DPlan(nx=nx, ny=ny, nz=nz, npd=NPD, nt=10, dx=TTI_DX, dy=TTI_DX, dz=TTI_DX, dt=TTI_DT,
                        favg=TTI_FAVG, fsx=nx // 2, fsy=ny // 2, fsz=1, mode="fast")
    plan.set_model(v, e, d)
    plan.set_tilt(th, ph)
    plan.time_steps(max(3, args.warmup))
    nsteps = max(10, 10 * args.steps)
    ms = plan.time_steps(nsteps) / nsteps
    plan.close()
    pts = (nx + 2 * NPD - 8) * (ny + 2 * NPD - 8) * (nz + 2 * NPD - 8)
    peak, peak_kind = measured_peak()
    achieved = pts * TTI_BYTES_PER_PT / (ms / 1000) / 1e9
    cpu = None
    if not args.no_cpu:
        from oracle import orc
        orc.build(with_ref=False)
        n = 120
        cv, ce, cd, cth, cph = (a.cpu().numpy() for a in tti_model((n, n, n), seed=7))
        t0 = time.perf_counter()
        orc.fd3d(cv, ce, cd, theta=cth, phi=cph, npd=20, nt=10, dx=TTI_DX, dy=TTI_DX, dz=TTI_DX,
                 dt=np.float32(TTI_DT), favg=TTI_FAVG, pfac=10.0, fsx=n // 2, fsy=n // 2, fsz=1)
        sec = time.perf_counter() - t0
        cpu = {"value": (n + 40 - 8) ** 3 * 10 / sec / 1e9, "unit": "Gpt/s", "cores": os.cpu_count(),
               "kind": "port", "sample": "10 steps of 120^3 + 20 sponge, oracle FP32 TTI restatement, OpenMP"}
    print(json.dumps({"case": "tti", "metric": "grid-pt updates/s", "value": pts / (ms / 1000) / 1e9,
                      "unit": "Gpt/s", "ms_per_step": ms,
                      "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                   "frac": achieved / peak, "peak_kind": peak_kind,
                                   "unit_of_work": "one time step (%d updates, %d B each)" % (pts, TTI_BYTES_PER_PT)},
                      "config": {"workload": "3D TTI step, %dx%dx%d (+40 sponge) at 12.5 m, dt 0.8 ms, tilt "
                                             "0-45 deg, azimuth 0-360 deg (smooth seeded fields)" % (nx, ny, nz)},
                      "cpu_baseline": cpu, "dtype": "f32", "data": "synthetic"}), flush=True)


def run_tti_rtm_case(args):
    """3D TTI RTM on the 600x600x400 (+40 sponge) medium at 12.5 m, 3500
    steps, 12 Hz, a 300x300 receiver grid at 2-node spacing recording and
    taking the record back (--all-nodes: every surface node, the 3D RTM
    program's receivers): plain checkpoint
    recompute (full wavefield every K steps, segments re-propagated; the
    stored-snapshot image bit for bit) against snapshots every 4 steps
    through the learned codec trained on TTI snapshots from the solver.
    `--shots` shots back to back (sources spread along x); shots/hour of
    both and the learned image's error against the plain one (the image
    the codec is measured against).  The reference programs' boundary
    re-propagation is not that image here: it diverges on the TTI medium."""
    import torch

    import geophysics_gb300 as geo
    from geophysics_gb300 import build as B
    B.build()
    ny, nx, nz = TTI_SHAPE
    v, e, d, th, ph = tti_model(TTI_SHAPE)
    codec, tinfo = train_codec(geo, args.train_iters, tti=True)
    rk = dict(npd=NPD, dx=TTI_DX, dy=TTI_DX, dz=TTI_DX, dt=TTI_DT, favg=TTI_FAVG, fsx=nx // 2 - 100, fsy=ny // 2,
              dsx=200 // max(1, args.shots - 1) if args.shots > 1 else 0, fsz=1, mute_tt=70, laplace=True,
              mode="fast", theta=th, phi=ph, nt=args.nt, ns=args.shots, snap_every=4,
              receivers=None if args.all_nodes else (0, 2, nx // 2, 0, 2, ny // 2))

    def timed(**kw):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = geo.rtm3d(v, e, d, **rk, **kw)
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    plain, tp = timed(method="checkpoint")
    # two escape settings: (block error threshold, escaped-block budget)
    out = {}
    for name, tol, budget in (("learned", 0.02, args.escape), ("learned_tight", 0.01, 3 * args.escape)):
        codec.set_escape(tol, budget)
        b0, e0 = codec.stats()
        img, sec = timed(method="learned", codec=codec)
        b1, e1 = codec.stats()
        out[name] = (img, sec, (e1 - e0) / max(1, b1 - b0), tol, budget)

    def rel(a, b):
        a, b = a[0].double(), b[0].double()
        return float((a - b).norm() / b.norm())

    print(json.dumps({"case": "tti-rtm", "metric": "3D TTI RTM shots/hr, learned snapshot codec vs plain "
                                                   "checkpoint recompute", "grid": [nx, ny, nz], "sponge": NPD,
                      "nt": args.nt, "shots": args.shots, "snap_every": 4,
                      "receivers": "every surface node" if args.all_nodes else
                      "%dx%d grid at 2-node spacing" % (nx // 2, ny // 2),
                      "shots_per_hr": dict({"checkpoint": args.shots * 3600.0 / tp},
                                           **{k: args.shots * 3600.0 / o[1] for k, o in out.items()}),
                      "seconds": dict({"checkpoint": tp}, **{k: o[1] for k, o in out.items()}),
                      "speedup_vs_plain": {k: tp / o[1] for k, o in out.items()},
                      "image_rel_l2_vs_plain": {k: rel(o[0], plain) for k, o in out.items()},
                      "image": "Laplacian-filtered, illumination-divided",
                      "compression": {k: {"escape_tol": o[3], "escape_budget": o[4], "escaped_block_frac": o[2],
                                          "ratio": 16384 / (1024 + 4 + 4 + o[2] * 8192)} for k, o in out.items()},
                      "training": tinfo, "dtype": "f32 propagation, bf16 codec", "data": "synthetic"}), flush=True)


def run_rtm_methods_case(args):
    """Launch-list case: each RTM method of `--methods` for `--nt` steps on
    the 512x512x384 grid (untrained codec: the timing does not depend on the
    weights), then 45 bare steps of the same grid."""
    import torch

    import geophysics_gb300 as geo
    nx, ny, nz = 512, 512, 384
    vp, eps, dl = make_model(seed=4, device="cuda", shape=(ny, nx, nz))
    rk = dict(npd=NPD, dx=DX, dy=DX, dz=DX, dt=DT, favg=FAVG, fsx=nx // 2, fsy=ny // 2, fsz=1, mute_tt=70,
              laplace=False, mode="fast", sv=1, nt=args.nt)
    codec = geo.Codec(seed=1)
    out = {}
    for m in args.methods.split(","):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        geo.rtm3d(vp, eps, dl, method=m, snap_every=4, codec=codec, **rk)
        torch.cuda.synchronize()
        out[m] = time.perf_counter() - t0
    plan = geo.FD3DPlan(nx=nx, ny=ny, nz=nz, npd=NPD, nt=10, dx=DX, dy=DX, dz=DX, dt=DT, favg=FAVG, fsx=nx // 2,
                        fsy=ny // 2, fsz=1, mode="fast")
    plan.set_model(vp, eps, dl)
    plan.time_steps(5)
    out["bare_step_ms"] = plan.time_steps(40) / 40
    plan.close()
    print(json.dumps({"case": "rtm-methods", "grid": [nx, ny, nz], "nt": args.nt, "seconds": out}), flush=True)


def run_fd2d_case(args):
    """2D VTI FD, one shot, with the CPU program's arithmetic (CPU_vti2dfd):
    401x401 at 10 m, dt 1 ms, 2000 steps, 50-cell sponge, 20 Hz Ricker at
    (200, 5), every surface node recorded at z = 5; 5 flat seeded layers.
    The working set (~15 fields of 1 MB) stays in L2: the figure is grid-point
    updates per second, not an HBM fraction.  cpu: the oracle's restatement
    of the same shot on one host core (sample: 200 steps)."""
    import numpy as np
    import torch

    import geophysics_gb300 as geo
    from geophysics_gb300 import media
    from geophysics_gb300 import build as B
    B.build()
    nx = nz = 401
    npd, nt = 50, 2000
    v, e, d = media.layered_vti(nx, nz, seed=1)
    kw = dict(npd=npd, nt=nt, dx=10.0, dz=10.0, dt=1e-3, favg=20.0, fs=200, zs=5, variant="cpu", rec_iz=npd + 4)
    tv, te, td = (torch.from_numpy(a).cuda() for a in (v, e, d))
    for _ in range(args.warmup):
        geo.fd2d_shot(tv, te, td, **kw)
    torch.cuda.synchronize()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        geo.fd2d_shot(tv, te, td, **kw)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    t_host = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        geo.fd2d_shot(v, e, d, **kw)
        t_host.append(time.perf_counter() - t0)
    upd = (nx + 2 * npd - 8) * (nz + 2 * npd - 8) * nt
    cpu = None
    if not args.no_cpu:
        from oracle import orc
        orc.build(with_ref=False)
        ns = 200
        t0 = time.perf_counter()
        orc.fd2d(v, e, d, npd=npd, nt=ns, dx=10.0, dz=10.0, dt=np.float32(1e-3), favg=20.0, pfac=10.0, fs=200, zs=5,
                 rec_iz=npd + 4)
        dt = time.perf_counter() - t0
        cpu = {"value": (nx + 2 * npd - 8) * (nz + 2 * npd - 8) * ns / dt / 1e9, "unit": "Gpt/s", "cores": 1,
               "kind": "port", "sample": "200 of the 2000 steps, CPU program arithmetic, one core"}
    med = statistics.median(times)
    print(json.dumps({"case": "fd2d", "metric": "grid-pt updates/s", "value": upd / med / 1e9, "unit": "Gpt/s",
                      "ms_per_shot": 1000 * med, "e2e_ms_per_shot": 1000 * statistics.median(t_host),
                      "config": {"workload": "2D VTI FD 401x401, 2000 steps, dt 1 ms, 50 sponge, CPU_vti2dfd "
                                             "arithmetic"}, "cpu_baseline": cpu, "dtype": "f32"}), flush=True)


def run_rtm2d_case(args):
    """Batched 2D RTM: 128 shots on a 2401x601 layered + random-field model
    (10 m), aperture widths odd in 401..1199 (seeded), sources evenly over
    x = 601..1801, 3000 steps at dt 1 ms, 20 Hz, every node of the window
    recorded; per-shot image, stacked, adjoint Laplacian.  One persistent
    launch per half-step over all shots' tiles, the time loop in CUDA graphs,
    tiles from the autotuner.  cpu: the oracle's MPI-program restatement of
    one shot on one core (sample: 300 steps of the widest window)."""
    import numpy as np
    import torch

    import geophysics_gb300 as geo
    from geophysics_gb300 import media
    from geophysics_gb300 import build as B
    B.build()
    nx, nz, npd, nt, ns = 2401, 601, 50, args.nt, args.shots
    v, e, d = media.layered_random_vti(nx, nz, seed=3)
    rng = np.random.default_rng(3)
    widths = (rng.integers(200, 600, ns) * 2 + 1).astype(int)
    xs = np.round(np.linspace(601, 1801, ns)).astype(int)
    kw = dict(npd=npd, nt=nt, dx=10.0, dz=10.0, dt_ms=1.0, favg=20.0, pfac=10.0, zs=5, shot_x=xs, shot_nxs=widths)
    tv, te, td = (torch.from_numpy(a).cuda() for a in (v, e, d))
    geo.rtm2d_batch(tv, te, td, **dict(kw, nt=100))  # warm-up: autotune + graphs on a short run
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    img = geo.rtm2d_batch(tv, te, td, **kw)
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    # the fast mode (the program's double-precision chains in FP32), against the exact image
    geo.rtm2d_batch(tv, te, td, **dict(kw, nt=100, mode="fast"))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fimg = geo.rtm2d_batch(tv, te, td, **dict(kw, mode="fast"))
    torch.cuda.synchronize()
    fsec = time.perf_counter() - t0
    a, b = img.double(), fimg.double()
    na = float(torch.linalg.vector_norm(a))
    # short runs can end before any reflection reaches the image (zero norm)
    fast = {"seconds": fsec, "shots_per_hr": ns * 3600.0 / fsec,
            "image_rel_l2_vs_exact": float(torch.linalg.vector_norm(b - a)) / na if na > 0 else None}
    upd = sum((int(w) + 2 * npd - 8) * (nz + 2 * npd - 8) for w in widths) * nt * 3
    cpu = None
    if not args.no_cpu:
        from oracle import orc
        orc.build(with_ref=False)
        k = int(np.argmax(widths))
        s_nt = 300
        t1 = time.perf_counter()
        orc.rtm2d_mpi_shot(v, e, d, npd=npd, nt=s_nt, dx=10.0, dz=10.0, dt_ms=1.0, favg=20.0, pfac=10.0,
                           fs_sxd=int(xs[k]), ds_sxd=0, zs_sxd=5, is_=1, nxs=int(widths[k]))
        dt = time.perf_counter() - t1
        cu = (int(widths[k]) + 2 * npd - 8) * (nz + 2 * npd - 8) * s_nt * 3
        cpu = {"value": cu / dt / 1e9, "unit": "Gpt/s", "cores": 1, "kind": "port",
               "sample": "one shot (the widest window), 300 of 3000 steps, MPI-program arithmetic, one core",
               "shots_per_hr_extrapolated": 3600.0 / (dt * nt / s_nt * upd / ns / 3 / cu * 3)}
    print(json.dumps({"case": "rtm2d", "metric": "shots/hr", "value": ns * 3600.0 / sec, "unit": "shots/hr",
                      "seconds": sec, "grid_pt_updates_per_s": upd / sec / 1e9,
                      "image_finite": bool(torch.isfinite(torch.as_tensor(img)).all()), "fast_mode": fast,
                      "config": {"workload": "%d-shot batched 2D VTI RTM, 2401x601, widths 401-1199, %d steps"
                                             % (ns, nt)},
                      "cpu_baseline": cpu, "dtype": "f32"}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--case", default="full", choices=["full", "small", "traffic", "rtm-learned", "rtm-methods", "fd2d", "rtm2d",
                                                      "tti", "tti-rtm", "codec", "prog2d"],
                    help="small / traffic: ncu profiling cases; rtm-learned: the learned-codec RTM comparison")
    ap.add_argument("--grid", type=int, default=None, help="small (192 by default), tti (600x600x400 by "
                                                           "default): cube edge, for profiling cases")
    ap.add_argument("--sponge", type=int, default=40, help="small: sponge width")
    ap.add_argument("--nt", type=int, default=None, help="rtm-learned, rtm2d (default 3000), tti-rtm (default "
                    "3500): time steps")
    ap.add_argument("--shots", type=int, default=None, help="rtm2d: shots in the batch (default 128, the "
                    "workload's); tti-rtm: shots back to back (default 8, the workload's)")
    ap.add_argument("--all-nodes", action="store_true", help="tti-rtm: every surface node records (default: the "
                    "300x300 grid at 2-node spacing)")
    ap.add_argument("--train-iters", type=int, default=16000, help="rtm-learned: codec training steps")
    ap.add_argument("--escape", type=float, default=0.03, help="rtm-learned: escaped-block budget")
    ap.add_argument("--methods", default="boundary,learned", help="rtm-methods: methods to run")
    args = ap.parse_args()
    if args.case == "fd2d":
        run_fd2d_case(args)
        return
    if args.case == "codec":
        run_codec_case(args)
        return
    if args.case == "prog2d":
        run_prog2d_case(args)
        return
    if args.shots is None:
        args.shots = {"rtm2d": 128, "tti-rtm": 8}.get(args.case, 1)
    if args.nt is None:
        args.nt = TTI_NT if args.case == "tti-rtm" else 3000
    if args.case == "rtm2d":
        run_rtm2d_case(args)
        return
    if args.case == "tti":
        run_tti_case(args)
        return
    if args.case == "tti-rtm":
        run_tti_rtm_case(args)
        return
    if args.case == "rtm-methods":
        run_rtm_methods_case(args)
        return
    if args.case == "rtm-learned":
        run_rtm_learned_case(args)
        return
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
