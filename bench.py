"""Benchmark of the amdat_gb300 hot path on GB300.

Headline workload (the reference's coherent-ISF + static S(k) configuration):
binary 80:20 mixture, N = 32000 atoms, cubic box L = 33.6, 400 linear frames,
Gaussian random-walk steps sigma = 0.03 per frame (seeded, synthetic).  One
step = the whole coherent-ISF command: rho(k,t) for every half-space
integer-lattice vector with |k| <= 20 (2,562,052 vectors; the other half
space is the complex conjugate) over all 400 frames, the coherent F(k,t)
correlator over all 79,801 time pairs of the linear scheme in 0.1-wide shells,
and S(k).  Metric: atom*k/s = N * frames * vectors / step time.

Secondary workload (the MSD + self-ISF configuration): N = 4000, L = 16.8,
blocked-exponential 10 x 27 frames (base 1.3, unit 0.005), steps
0.05*sqrt(dt); one step = MSD, NGP moments and F_s at all lattice vectors with
|k| in [7.0, 7.2]; metric atom*time-pairs/s.

Both report the mixed-precision engine against its plain FP64 GPU path.
`--impl reference` times the CPU restatement of the reference algorithm on
the host cores instead (the reference binary itself is x86-only here).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "atom·time-pairs/s (MSD+Fs) & atom·k/s (rho_k): mixed vs FP64 plain, 1 GB300"
PEAKS_FILE = os.path.join(HERE, "MEASURED_PEAKS.json")
FP32_LANES_PER_SM = 128
# DRAM bytes (read + write) per frame of one rhok_tc_kernel launch on the headline
# lattice (N=32000, |k|<=20, L=33.6), from one ncu capture of a 2-frame launch of
# this kernel (941.9 MB read + 42.7 MB written).  Every stream of the launch is per
# frame (X/Y phase tables, Z operands, rho rows), so a launch over f frames moves f
# times this.
TC_DRAM_BYTES_PER_FRAME = (941.943e6 + 42.651e6) / 2
# DRAM bytes (read + write) of one launch of the per-list MSD + NGP plan over the 64
# nested lists, from one ncu capture of disp_mixed_kernel on that workload
PERLIST_DRAM_BYTES = 2.33e9
# MUFU (special-function unit) results per clock per SM: 4 per sub-partition
MUFU_PER_SM_CLK = 16


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def isf_workload(frames: int = 400, n_atoms: int = 32000):
    from amdat_gb300 import synth
    scheme = synth.TimeScheme.linear(frames, 1.0)
    traj = synth.random_walk(n_atoms, 33.6, scheme, 0.03, seed=2, type_fractions=(0.8, 0.2),
                             time_scaled=False)
    return traj, scheme, dict(kmax=20.0, dk=0.1, period=33.6)


def msd_workload():
    from amdat_gb300 import synth
    scheme = synth.TimeScheme.exponential(10, 27, 1.3, 0, 0, 0.005)
    traj = synth.random_walk(4000, 16.8, scheme, 0.05, seed=1)
    return traj, scheme


def batched_workload():
    """64 lists, log-uniform sizes 100..50000, nested prefixes of one random
    permutation of a 200000-atom walk (12 blocks x 30 frames, base 1.25)."""
    from amdat_gb300 import synth
    scheme = synth.TimeScheme.exponential(12, 30, 1.25, 0, 0, 0.005)
    traj = synth.random_walk(200000, 61.9, scheme, 0.05, seed=4)
    rng = np.random.default_rng(4)
    sizes = np.sort(np.exp(rng.uniform(np.log(100), np.log(50000), 64)).astype(np.int64))
    perm = rng.permutation(200000)
    return traj, scheme, sizes, perm


def reference_shells(ms):
    z = np.load(os.path.join(HERE, "tests", "golden", "qvectors3d.npz"))
    n, off = z["n"].astype(np.int32), z["offsets"]
    kv = np.concatenate([n[off[m]:off[m + 1]] for m in ms])
    o = np.concatenate([[0], np.cumsum([off[m + 1] - off[m] for m in ms])]).astype(np.int32)
    return kv, o


def tc_tile_entries(period, kmax):
    """Entries (complex rows x nz columns) the tensor-core tiling computes per
    atom and frame: 8x8 (nx, ny) squares x nz windows (one window of the smallest
    multiple of 16 covering 0..nmax, or windows of 128), each tile trimmed to a
    multiple of 16 columns covering its rows' nz extent in the window."""
    R = kmax * period / (2 * np.pi)
    nmax = int(np.floor(R))
    nzw = min(128, (nmax + 1 + 15) // 16 * 16)
    total = 0
    for x0 in range(-nmax, nmax + 1, 8):
        for y0 in range(-nmax, nmax + 1, 8):
            nx = np.arange(x0, x0 + 8)[:, None]
            ny = np.arange(y0, y0 + 8)[None, :]
            r2 = R * R - nx.astype(float) ** 2 - ny.astype(float) ** 2
            ok = (np.abs(nx) <= nmax) & (np.abs(ny) <= nmax) & (r2 >= 0)
            if not ok.any():
                continue
            zmax = int(np.floor(np.sqrt(r2[ok]).max()))
            for zb in range(0, zmax // nzw + 1):
                last = min(zmax - zb * nzw, nzw - 1)
                total += 64 * ((last + 1 + 15) // 16 * 16)
    return total


def lattice_shell(period, kmin, kmax):
    nmax = int(np.ceil(kmax * period / (2 * np.pi))) + 1
    r = np.arange(-nmax, nmax + 1)
    g = np.stack(np.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3)
    k = 2 * np.pi * np.linalg.norm(g, axis=1) / period
    return g[(k >= kmin) & (k <= kmax)].astype(np.int32)


def lattice_halfspace(period, kmax):
    nmax = int(np.floor(kmax * period / (2 * np.pi)))
    r = np.arange(-nmax, nmax + 1)
    g = np.stack(np.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3)
    n2 = (g.astype(np.float64) ** 2).sum(1)
    R = kmax * period / (2 * np.pi)
    x, y, z = g[:, 0], g[:, 1], g[:, 2]
    half = (z > 0) | ((z == 0) & ((y > 0) | ((y == 0) & (x > 0))))
    return g[(n2 <= R * R) & half].astype(np.int32)


# ---------------------------------------------------------------------------
# environment: ranks, clocks, peaks
# ---------------------------------------------------------------------------
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    """Host barrier over the ranks (no-op at one rank)."""
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x):
    """The largest of each rank's x (a step time): the job ends with its slowest rank."""
    if pg is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world, ms):
    """Whole-job throughput: every rank processes units_per_rank in a step whose
    time is the maximum over ranks (ms)."""
    return units_per_rank * world / (ms / 1e3)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.samples.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if s[3 + i].lower().startswith("active")})
        pw = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "power_w_max": max(pw) if pw else None, "samples": len(self.samples)}


def measured_peaks():
    try:
        with open(PEAKS_FILE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# ---------------------------------------------------------------------------
# CPU baseline (restatement of the reference algorithm, all host threads)
# ---------------------------------------------------------------------------
def cpu_rhok_sample(traj, vectors, threads, target_s=12.0):
    """rho(k) of the middle frame over a random vector sample, FP64, OpenMP over
    vectors (the reference's Wave_Density loop restated); grows the sample until
    it takes about target_s / 4.  Returns (rate, description, seconds, sample
    indices into vectors, rho [1][sample][2])."""
    from oracle import oracle as orc
    wrapped = traj.wrapped()
    rng = np.random.default_rng(0)
    nk = 2000
    frames = np.array([traj.n_frames // 2], np.int32)
    while True:
        idx = np.sort(rng.choice(len(vectors), size=min(nk, len(vectors)), replace=False))
        t0 = time.perf_counter()
        out = orc.rhok_parallel(wrapped, frames, vectors[idx], float(traj.box[0]), threads)
        dt = time.perf_counter() - t0
        units = traj.n_atoms * len(idx)
        if dt >= target_s / 4 or nk >= len(vectors):
            return (units / dt, f"1 frame x {len(idx)} random vectors x {traj.n_atoms} atoms", dt,
                    idx, out)
        nk = int(min(len(vectors), nk * max(2.0, (target_s / 4) / max(dt, 1e-3))))


def cpu_disp_sample(traj, scheme, shell, threads):
    """MSD and F_s of every time pair and atom, FP64 (OpenMP over atoms).
    Returns (rate, description, seconds, per-gap sum |dr|^2, per-gap F_s sums)."""
    from oracle import oracle as orc
    s = orc.scheme(scheme)
    t0 = time.perf_counter()
    d2, fs = orc.disp_fs_parallel(s, traj.unwrapped, shell, float(traj.box[0]), threads)
    dt = time.perf_counter() - t0
    npairs = len(orc.pairs(s, 0)[0])
    return (npairs * traj.n_atoms / dt, f"all {npairs} time pairs x {traj.n_atoms} atoms, {len(shell)} vectors",
            dt, d2, fs)


def write_qvector_files(directory):
    """The reference's q-vector tables as its text files qvector.NNN (shell m in file m + 2)."""
    z = np.load(os.path.join(HERE, "tests", "golden", "qvectors3d.npz"))
    n, off = z["n"], z["offsets"]
    d = os.path.join(directory, "qvectors3d")
    os.makedirs(d, exist_ok=True)
    for m in range(len(off) - 1):
        with open(os.path.join(d, f"qvector.{m + 2:03d}"), "w") as f:
            f.writelines(f"   {float(v[0]):.7e}   {float(v[1]):.7e}   {float(v[2]):.7e}\n" for v in n[off[m]:off[m + 1]])
    return os.path.join(d, "qvector")


def cli_bench():
    """The drop-in path end to end: an AMDAT input script through the command-line
    driver on the MSD workload (N=4000, 271 frames, exponential 10 x 27 base 1.3):
    custom-dump parse, upload, msd, ngp, isfs (reference shell 36) and vhs, output
    files written.  A second script with the system block alone times ingestion."""
    import tempfile
    from amdat_gb300 import synth
    traj, scheme = msd_workload()
    cli = os.path.join(HERE, "amdat_gb300", "_lib", "amdat_gb300")
    with tempfile.TemporaryDirectory() as tmp:
        dump = os.path.join(tmp, "traj.dump")
        synth.write_custom_dump(traj, dump)
        env = dict(os.environ, AMDAT_QVECTORS=write_qvector_files(tmp))
        header = synth.system_header(traj, dump)
        script = ("create_list all\nall\nmsd ./msd.dat\nlist all\nngp ./ngp.dat\nlist all\n"
                  "isfs ./isfs.dat 36 36 xyz 0\nlist all\nvhs ./vhs.dat 2.0 100\nlist all\n")
        times = {}
        for tag, text in (("ingest", header + "create_list all\nall\n"), ("script", header + script)):
            path = os.path.join(tmp, f"{tag}.in")
            with open(path, "w") as f:
                f.write(text)
            best = None
            for _ in range(3):
                t0 = time.perf_counter()
                r = subprocess.run([cli, "-i", path], cwd=tmp, env=env, capture_output=True, text=True)
                dt = time.perf_counter() - t0
                if r.returncode != 0:
                    raise RuntimeError(f"amdat_gb300 CLI failed: {r.stderr[-500:]}")
                best = dt if best is None else min(best, dt)
            times[tag] = best
        mb = os.path.getsize(dump) / 1e6
    npairs = 316
    return dict(dump_mb=mb, ingest_s=times["ingest"], script_s=times["script"],
                analyses_s=times["script"] - times["ingest"], atoms=traj.n_atoms, frames=traj.n_frames,
                units=float(traj.n_atoms) * npairs)


REF_SHELLS = 20  # the reference arm's q-vector shells 0..20 (2,843 vectors)
REF_FRAMES = 2   # frames of the headline walk in the reference arm's sample


def reference_isf_sample(binary, threads, tmp):
    """The reference program's own coherent-ISF command on a bounded sample of the
    headline workload: the first REF_FRAMES frames of the N=32000, L=33.6 walk
    (custom dump), `isf ... auto symmetric xyz 0 0 REF_SHELLS` over the list of
    all atoms, i.e. Wave_Density::listkernel over every atom, frame and vector of
    the reference's q-vector shells 0..REF_SHELLS, then the correlator.  Returns
    a closure timing one run (seconds of the command: the run with the command
    minus the best of three runs of the same system block without it) and the
    sample's atom*k units."""
    from amdat_gb300 import synth
    traj, _, _ = isf_workload(REF_FRAMES)
    dump = os.path.join(tmp, "traj.dump")
    synth.write_custom_dump(traj, dump)
    header = synth.system_header(traj, dump)
    z = np.load(os.path.join(HERE, "tests", "golden", "qvectors3d.npz"))
    n_vec = int(z["offsets"][REF_SHELLS + 1])
    scripts = {"header": header + "create_list all\nall\n",
               "isf": header + f"create_list all\nall\nisf ./isf.dat auto symmetric xyz 0 0 {REF_SHELLS}\nlist all\n"}
    for k, text in scripts.items():
        with open(os.path.join(tmp, f"{k}.in"), "w") as f:
            f.write(text)

    def run(tag):
        t0 = time.perf_counter()
        r = subprocess.run([binary, "-n", str(threads), "-i", f"{tag}.in"], cwd=tmp,
                           capture_output=True, text=True)
        dt = time.perf_counter() - t0
        if r.returncode != 0:
            raise RuntimeError(f"reference AMDAT failed: {(r.stdout + r.stderr)[-500:]}")
        return dt

    base = min(run("header") for _ in range(3))
    units = float(traj.n_atoms) * REF_FRAMES * n_vec
    desc = (f"reference AMDAT binary (built here from its sources), `isf ... auto symmetric xyz 0 0 "
            f"{REF_SHELLS}`: {REF_FRAMES} frames x {n_vec} q-vectors (shells 0..{REF_SHELLS}) x "
            f"{traj.n_atoms} atoms; command time = run - system-block-only run ({base:.2f} s, best of 3)")
    return (lambda: run("isf") - base), units, desc


def run_reference(args):
    """The reference arm: the reference AMDAT program's own CPU path (its `isf`
    command) timed on this machine's host cores, on rank 0 only.  When its
    sources are not available here, the oracle's FP64 restatement of the same
    loop stands in (kind "port")."""
    import tempfile
    world, rank, local, pg = dist_setup()
    if rank != 0:
        return
    from oracle import build_oracle
    threads = os.cpu_count() or 1
    binary, why = None, ""
    try:
        binary = build_oracle.build_reference()
        if binary is None:
            why = "reference sources not present (baseline/_ref/src or AMDAT_REFERENCE)"
    except Exception as e:  # a failed build falls back to the restatement
        why = f"reference build failed: {str(e)[-200:]}"
    config = {"workload": "coherent ISF + S(k): rho_k(t), N=32000 (80:20), L=33.6, linear frames of a "
                          "sigma=0.03 random walk; the reference's Wave_Density loop over atoms x vectors"}
    if binary is not None:
        with tempfile.TemporaryDirectory() as tmp:
            one, units, desc = reference_isf_sample(binary, threads, tmp)
            for _ in range(args.warmup):
                one()
            secs = [one() for _ in range(args.steps)]
        dt = statistics.median(secs)
        value = units / dt
        kind, cores = "reference", 1
        note = (f"the reference is run with -n {threads}; its Wave_Density and correlator loops have no "
                "OpenMP, so one core does the work. Work is linear in atoms x frames x vectors, so the "
                "rate carries to the full 400-frame workload (extrapolated).")
    else:
        build_oracle.build_lib()
        traj, scheme, lat = isf_workload()
        vectors = lattice_halfspace(lat["period"], lat["kmax"])
        rate, desc, dt, _, _ = cpu_rhok_sample(traj, vectors, threads,
                                               target_s=4.0 * max(1, 12 // max(args.steps, 1)))
        vals = []
        for _ in range(args.warmup):
            cpu_rhok_sample(traj, vectors, threads, target_s=dt * 4)
        for _ in range(args.steps):
            vals.append(cpu_rhok_sample(traj, vectors, threads, target_s=dt * 4)[0])
        value = statistics.median(vals)
        kind, cores = "port", threads
        note = f"{why}; the oracle's FP64 restatement of the reference loop (OpenMP over vectors) instead"
    config["sample_per_step"] = desc
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "atom·k/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if kind == "reference" else "f64", "data": "synthetic",
            "config": config,
            "cpu_baseline": {"value": value, "unit": "atom·k/s", "cores": cores, "kind": kind,
                             "sample": desc},
            "e2e": {"value": value, "unit": "atom·k/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": note}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def structure_bench(torch, stream, device, args, n_atoms=100000, box=48.9, frames=10):
    """Differentiable structure: loss = sum_r (g(r) - g_t(r))^2 + sum_k (S(k) - S_t(k))^2,
    g Gaussian-smoothed (sigma 0.02, 400 bins to 4.0), S(k) over all half-space
    lattice k with |k| <= 12 (shells of 0.1), N=100000, L=48.9, 10 frames of a
    random walk; targets from a second seed.  A step is one loss + gradient
    evaluation through the libtorch autograd functions (forward kernels, both
    adjoints)."""
    from amdat_gb300 import autograd as AG
    from amdat_gb300 import build, synth
    build.build_torch_ext()
    ext = AG.ext()
    sc = synth.TimeScheme.linear(frames, 1.0)
    B = [box, box, box]
    pos_np = synth.random_walk(n_atoms, box, sc, 0.1, seed=7, time_scaled=False).wrapped()
    tgt_np = synth.random_walk(n_atoms, box, sc, 0.1, seed=8, time_scaled=False).wrapped()
    dev = torch.device("cuda", device)
    pos_host = torch.from_numpy(np.ascontiguousarray(pos_np)).pin_memory()
    grad_host = torch.empty_like(pos_host).pin_memory()
    loss_host = torch.empty((), dtype=torch.float64).pin_memory()
    with torch.no_grad():
        tgt = torch.from_numpy(np.ascontiguousarray(tgt_np)).to(dev)
        g_t = AG.g_of_r(AG.gsmooth(tgt, B), n_atoms, frames, B)
        s_t = AG.s_of_k(AG.structure_factor_raw(tgt, B), n_atoms, frames)
    pos = pos_host.to(dev)

    def step(p):
        p = p.detach().requires_grad_(True)
        loss, _, _ = AG.structure_loss(p, B, g_t, s_t)
        loss.backward()
        return loss.detach(), p.grad

    for _ in range(max(args.warmup, 1)):
        step(pos)
    torch.cuda.synchronize()
    ext.profile_reset(True, device)
    n0 = ext.launch_count(device)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record(stream)
    for _ in range(args.steps):
        step(pos)
    ev[1].record(stream)
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[1]) / args.steps
    launches = (ext.launch_count(device) - n0) // args.steps
    kern = {}
    for name in ("gsmooth_kernel", "gsmooth_adjoint_kernel", "rhok_tc_kernel", "rhok_lattice_kernel",
                 "sk_frames_kernel", "sk_adjoint_columns_kernel", "sk_adjoint_tc_kernel"):
        n, t = ext.profile_kernel(name, device)
        if n:
            kern[name] = t / args.steps
    ext.profile_reset(False, device)
    # end to end: positions from pinned host memory, loss and gradient back
    ev[0].record(stream)
    for _ in range(args.steps):
        loss, grad = step(pos_host.to(dev, non_blocking=True))
        grad_host.copy_(grad, non_blocking=True)
        loss_host.copy_(loss, non_blocking=True)
    ev[1].record(stream)
    torch.cuda.synchronize()
    e2e_ms = ev[0].elapsed_time(ev[1]) / args.steps
    kv, off = AG.lattice(pos, B)
    nk = int(kv.shape[0])
    pairs = frames * n_atoms * (n_atoms - 1) / 2.0
    fp32_peak = 2 * 128 * torch.cuda.get_device_properties(device).multi_processor_count * 2.07e9 / 1e12
    out = {
        "workload": f"differentiable structure: loss = sum (g - g_t)^2 + sum (S - S_t)^2, g Gaussian-"
                    f"smoothed (sigma 0.02, 400 bins to 4.0), S(k) over {nk} half-space lattice k with "
                    f"|k|<=12 (shells of 0.1), N={n_atoms}, L={box}, {frames} random-walk frames, "
                    f"targets from a second seed; one step = loss + gradient",
        "value": 1e3 / ms, "unit": "loss+gradient evaluations/s", "ms_per_step": ms,
        "e2e": {"value": 1e3 / e2e_ms, "unit": "loss+gradient evaluations/s",
                "h2d_bytes_per_step": int(pos_host.numel() * 4),
                "d2h_bytes_per_step": int(grad_host.numel() * 4 + 8), "ms_per_step": e2e_ms},
        "gpu_launches": int(launches),
        "kernel_ms_per_step": kern,
        "vectors": nk,
    }
    if "gsmooth_kernel" in kern:
        out["gsmooth_pairs_per_s"] = pairs / (kern["gsmooth_kernel"] / 1e3)
    if "gsmooth_adjoint_kernel" in kern:
        out["gsmooth_adjoint_ordered_pairs_per_s"] = 2 * pairs / (kern["gsmooth_adjoint_kernel"] / 1e3)
    if "sk_adjoint_tc_kernel" in kern:
        r = frames * n_atoms * nk / (kern["sk_adjoint_tc_kernel"] / 1e3)
        peak = measured_peaks().get("bf16_tflops_sustained", 1700.0)
        out["sk_adjoint_atom_k_per_s"] = r
        out["sk_adjoint_roofline"] = {
            "bound": "tensor", "achieved": 16 * r / 1e12, "peak": peak, "unit": "TFLOP/s",
            "frac": 16 * r / 1e12 / peak,
            "rule": "16 flops per atom x vector (one complex MAC for T and one for the nz-weighted T'); "
                    "the kernel issues 3 FP16 split passes over whole tiles; peak = measured sustained "
                    "bf16/fp16 dense rate"}
    if "sk_adjoint_columns_kernel" in kern:
        r = frames * n_atoms * nk / (kern["sk_adjoint_columns_kernel"] / 1e3)
        out["sk_adjoint_atom_k_per_s"] = r
        out["sk_adjoint_roofline"] = {
            "bound": "fp32", "achieved": 12 * r / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
            "frac": 12 * r / 1e12 / fp32_peak,
            "rule": "12 flops per atom x vector: Im(c e) (mul + fma = 3), shell sum (1), nz-weighted "
                    "sum (fma = 2), phase rotation (2 mul + 2 fma = 6); peak = 2 flops x 128 FP32 "
                    "lanes x SMs x 2.07 GHz"}
    return out


def isf_device_checks(torch, eng, E, d_rho, off, d_corr, d_pc, d_sk, N, T, shells=(20, 60, 120, 199)):
    """FP64 restatement on the device of the correlator and S(k) of a few whole
    shells, from the engine's own rho table of the timed workload: S(k) =
    <|rho|^2> / N over frames and the shell's vectors, F(k, gap) = mean over the
    gap's time pairs (the scheduler's own pair table) of the shell mean of
    Re rho(t0) Re rho(t1) + Im rho(t0) Im rho(t1), divided by N.  Returns the
    largest deviations relative to S(k)."""
    g, a, b = E.scheme_pairs(eng.scheme, 0, 1)
    dev = d_rho.device
    g_t = torch.from_numpy(g.astype(np.int64)).to(dev)
    a_t = torch.from_numpy(a.astype(np.int64)).to(dev)
    b_t = torch.from_numpy(b.astype(np.int64)).to(dev)
    G = d_corr.shape[0]
    corr = d_corr.double().cpu().numpy()
    pc = d_pc.cpu().numpy()
    sk = d_sk.double().cpu().numpy() / (N * T)
    worst_f, worst_s, used, pairs_match = 0.0, 0.0, [], True
    for m in shells:
        if m + 1 >= len(off) or off[m + 1] == off[m]:
            continue
        used.append(int(m))
        r = d_rho[:, int(off[m]):int(off[m + 1])].double()  # [T, V, 2]
        s_ref = float((r ** 2).sum(-1).mean()) / N
        worst_s = max(worst_s, abs(sk[m] - s_ref) / s_ref)
        acc = torch.zeros(G, dtype=torch.float64, device=dev)
        cnt = torch.zeros(G, dtype=torch.float64, device=dev)
        for c0 in range(0, len(g), 512):
            ta, tb, tg = a_t[c0:c0 + 512], b_t[c0:c0 + 512], g_t[c0:c0 + 512]
            prod = (r[ta] * r[tb]).sum(-1).mean(1)
            acc.index_add_(0, tg, prod)
            cnt.index_add_(0, tg, torch.ones_like(prod))
        pairs_match = pairs_match and bool((cnt.cpu().numpy().astype(np.int64) == pc).all())
        f_ref = (acc / cnt.clamp(min=1) / N).cpu().numpy()
        f_eng = corr[:, m] / (np.maximum(pc, 1) * N)
        worst_f = max(worst_f, float(np.abs(f_eng - f_ref).max()) / s_ref)
    return {"shells": used, "sk_worst_rel": worst_s, "isf_worst_rel_to_sk": worst_f,
            "pair_counts_match": pairs_match,
            "rule": "FP64 torch restatement on the device of S(k) and F(k,t) over whole shells, "
                    "from the engine's rho table of the timed workload"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--frames", type=int, default=400, help="frames of the headline workload")
    ap.add_argument("--only", default="", choices=["", "isf", "msd", "batched", "pairs", "structure", "cli",
                                                   "perlist", "shared", "bins"],
                    help="run one workload only (profiling)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--pair-frames", type=int, default=50,
                    help="frames of the RDF / van Hove workload (profiling runs use fewer)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    from amdat_gb300 import build
    from amdat_gb300 import engine as E

    world, rank, local, pg = dist_setup()
    torch.cuda.set_device(local)
    build.build()
    peaks = measured_peaks()
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    # a dedicated stream: the engine launches on it and the CUDA events below
    # are recorded on it (torch's default stream is the legacy NULL stream)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    eng = E.Engine(local)
    eng.set_stream(stream.cuda_stream)

    result = {}
    clocks = ClockSampler(local)
    if args.only in ("", "isf"):
        traj, scheme, lat = isf_workload(args.frames)
        T, N = traj.n_frames, traj.n_atoms
        eng.upload(traj.unwrapped, traj.box)
        eng.set_scheme(scheme)
        frames = np.arange(T, dtype=np.int32)
        h, nk, ns = eng.wave_density_lattice(0, lat["kmax"], lat["dk"], lat["period"], frames)
        kv, off = eng.wave_density_vectors(h, nk, ns)
        eng.wave_density_free(h)
        G = eng.n_timegaps
        d_corr = torch.empty((G, ns), dtype=torch.float64, device="cuda")
        d_pc = torch.empty(G, dtype=torch.int64, device="cuda")
        d_sk = torch.empty(ns, dtype=torch.float64, device="cuda")

        def step():
            hh, _, _ = eng.wave_density_lattice(0, lat["kmax"], lat["dk"], lat["period"], frames)
            eng.isf(hh, hh, off, out_device=(d_corr.data_ptr(), d_pc.data_ptr()))
            eng.structure_factor(hh, hh, off, out_device=d_sk.data_ptr())
            eng.wave_density_free(hh)

        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        barrier(pg)
        eng.profile_reset(True)
        l0 = eng.launch_count()
        clocks.start()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        clocks.stop()
        barrier(pg)
        ms = e0.elapsed_time(e1) / args.steps
        ms = max_over_ranks(pg, ms)
        launches = eng.launch_count() - l0
        kname = "rhok_tc_kernel"
        n_lat, ms_lat = eng.profile_kernel(kname)
        if n_lat == 0:
            kname = "rhok_lattice_kernel"
            n_lat, ms_lat = eng.profile_kernel(kname)
        n_isf, ms_isf = eng.profile_kernel("isf_lag_kernel")  # linear scheme: the lag kernel
        if n_isf == 0:
            n_isf, ms_isf = eng.profile_kernel("isf_pairs_kernel")
        eng.profile_reset(False)
        units = float(N) * T * nk
        value = job_rate(units, world, ms)
        # roofline of the dominant kernel: 8 algorithmic flops (one complex
        # multiply-accumulate) per atom*vector; the tensor-core kernel issues
        # 3 split-precision passes over whole tiles, reported as issued flops
        lat_ms = ms_lat / max(n_lat, 1) * n_lat / max(args.steps, 1)  # per step (launches = frame batches)
        flops = 8.0 * N * T * nk
        achieved = flops / (lat_ms / 1e3) / 1e12
        issued = None
        if kname == "rhok_tc_kernel":
            issued = 24.0 * N * T * tc_tile_entries(lat["period"], lat["kmax"]) / (lat_ms / 1e3) / 1e12
        clk = clocks.summary()
        fp32_peak_max = 2 * FP32_LANES_PER_SM * sm_count * float(peaks.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12
        # plain FP64 path on one frame of the same workload
        fr1 = np.array([T // 2], np.int32)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hp, _, _ = eng.wave_density_lattice(0, lat["kmax"], lat["dk"], lat["period"], fr1, precision=1)
        eng.synchronize()
        plain_s = time.perf_counter() - t0
        eng.wave_density_free(hp)
        plain_rate = float(N) * nk / plain_s
        # end to end through the C ABI: pinned host trajectory in, results out
        pinned = torch.empty((T, N, 3), dtype=torch.float32, pin_memory=True)
        pinned.numpy()[...] = traj.unwrapped
        corr_h = np.zeros((G, ns))
        sk_h = np.zeros(ns)

        def e2e_step():
            eng.upload_ptr(pinned.data_ptr(), T, N, traj.box)
            eng.set_scheme(scheme)
            hh, _, _ = eng.wave_density_lattice(0, lat["kmax"], lat["dk"], lat["period"], frames)
            c, pc = eng.isf(hh, hh, off)
            corr_h[...] = c
            sk_h[...] = eng.structure_factor(hh, hh, off)
            eng.wave_density_free(hh)

        e2e_step()
        torch.cuda.synchronize()
        barrier(pg)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        e2e_ms = max_over_ranks(pg, 1e3 * (time.perf_counter() - t0) / max(1, args.steps))
        del pinned
        # one more step whose results are kept and checked (outside every timed region):
        # the correlator and S(k) against an FP64 restatement on the device, and the
        # rho table's middle frame against the FP64 oracle in the CPU leg below
        hh, _, _ = eng.wave_density_lattice(0, lat["kmax"], lat["dk"], lat["period"], frames)
        d_rho = torch.empty((T, nk, 2), dtype=torch.float32, device="cuda")
        eng.wave_density_read(hh, T, nk, out_device=d_rho.data_ptr())
        eng.isf(hh, hh, off, out_device=(d_corr.data_ptr(), d_pc.data_ptr()))
        eng.structure_factor(hh, hh, off, out_device=d_sk.data_ptr())
        torch.cuda.synchronize()
        eng.wave_density_free(hh)
        checks = isf_device_checks(torch, eng, E, d_rho, off, d_corr, d_pc, d_sk, N, T)
        rho_mid = d_rho[T // 2].cpu().numpy()
        del d_rho
        result["isf"] = dict(
            value=value, ms=ms, launches=launches, nk=nk, ns=ns, T=T, N=N, kname=kname, issued=issued,
            lat_ms=lat_ms, n_lat=n_lat, steps=args.steps, isf_ms=ms_isf / max(n_isf, 1), achieved=achieved,
            fp32_peak_max=fp32_peak_max, clocks=clk, plain_rate=plain_rate,
            e2e=job_rate(units, world, e2e_ms), e2e_ms=e2e_ms,
            h2d=int(T * N * 3 * 4), d2h=int(G * ns * 8 + G * 8 + ns * 8),
            checks=checks, rho_mid=rho_mid, kv=kv)

    if args.only in ("", "msd"):
        mtraj, mscheme = msd_workload()
        shell = lattice_shell(16.8, 7.0, 7.2)
        off = np.array([0, len(shell)], np.int32)
        eng.upload(mtraj.unwrapped, mtraj.box)
        eng.set_scheme(mscheme)
        G = eng.n_timegaps
        d_out = [torch.zeros(G, dtype=torch.float64, device="cuda") for _ in range(2)]
        d_cnt = torch.zeros(G, dtype=torch.int64, device="cuda")
        d_fs = torch.zeros(G, dtype=torch.float64, device="cuda")

        def mstep(precision=0):
            eng.disp_device((d_out[0].data_ptr(), d_out[1].data_ptr(), d_cnt.data_ptr(),
                             d_fs.data_ptr(), 0), 0, shells=(shell, off), period=16.8,
                            precision=precision)

        for _ in range(max(3, args.warmup)):
            mstep()
        torch.cuda.synchronize()
        msteps = 50
        # the trajectory (13 MB) fits in L2: every timed step is bracketed by its own
        # events and L2 is flushed (a 256 MB write) between steps, outside the events
        flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
        eng.profile_reset(True)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(msteps)]
        for e0, e1 in evs:
            flush.fill_(1.0)
            e0.record(stream)
            mstep()
            e1.record(stream)
        torch.cuda.synchronize()
        mms = max_over_ranks(pg, sum(e0.elapsed_time(e1) for e0, e1 in evs) / msteps)
        n_d, ms_d = eng.profile_kernel("disp_mixed_kernel")
        eng.profile_reset(False)
        npairs = int(d_cnt.sum().item()) // mtraj.n_atoms
        munits = float(npairs) * mtraj.n_atoms
        m_out = dict(sum_d2=d_out[0].cpu().numpy(), sum_d4=d_out[1].cpu().numpy(),
                     cnt=d_cnt.cpu().numpy(), fs=d_fs.cpu().numpy())
        e0, e1 = evs[0]
        # the same pass as a prepared plan replayed from a CUDA graph (what repeated
        # analyses of one list use): no per-call table building or launch overhead
        mplan = eng.plan([0], shells=(shell, off), period=16.8, flags=E.PLAN_GRAPH | E.PLAN_AUTOTUNE)
        for _ in range(3):
            mplan.run()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(msteps):
            mplan.run()
        e1.record(stream)
        torch.cuda.synchronize()
        pms = max_over_ranks(pg, e0.elapsed_time(e1) / msteps)
        mplan.close()
        t0 = time.perf_counter()
        mstep(precision=1)
        eng.synchronize()
        mplain = munits / (time.perf_counter() - t0)
        # end to end through the C ABI: the trajectory from pinned host memory, the
        # per-gap sums back to the host, every step
        MT, MN = mtraj.n_frames, mtraj.n_atoms
        mpinned = torch.empty((MT, MN, 3), dtype=torch.float32, pin_memory=True)
        mpinned.numpy()[...] = mtraj.unwrapped

        def me2e():
            eng.upload_ptr(mpinned.data_ptr(), MT, MN, mtraj.box)
            eng.set_scheme(mscheme)
            return eng.disp(0, shells=(shell, off), period=16.8)

        for _ in range(3):
            me2e()
        t0 = time.perf_counter()
        for _ in range(msteps):
            me2e()
        me2e_ms = max_over_ranks(pg, 1e3 * (time.perf_counter() - t0) / msteps)
        del mpinned
        result["msd"] = dict(value=job_rate(munits, world, mms), ms=mms, kernel_ms=ms_d / max(n_d, 1),
                             plain=mplain, npairs=npairs, nvec=len(shell),
                             plan_value=job_rate(munits, world, pms), plan_ms=pms,
                             e2e=job_rate(munits, world, me2e_ms), e2e_ms=me2e_ms,
                             h2d=int(MT * MN * 12), d2h=int(G * (8 + 8 + 8 + 8)), out=m_out)

    if args.only in ("perlist", "shared"):
        # profiling aid: the batched workload's per-list (or membership-class
        # shared) MSD + NGP plan alone
        btraj, bscheme, sizes, perm = batched_workload()
        eng.upload(btraj.unwrapped[:, perm], btraj.box)
        eng.set_scheme(bscheme)
        nested = [eng.list(np.arange(n, dtype=np.int32)) for n in sizes]
        pflags = E.PLAN_AUTOTUNE | (E.PLAN_NO_SHARING if args.only == "perlist" else 0)
        plan = eng.plan(nested, flags=pflags)
        for _ in range(args.warmup):
            plan.run()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            plan.run()
        torch.cuda.synchronize()
        result["perlist"] = dict(ms=1e3 * (time.perf_counter() - t0) / max(args.steps, 1), info=plan.info(),
                                 plan=args.only)
        plan.close()

    if args.only == "bins":
        # profiling aid: the batched workload's 64-bin MSD pass alone
        btraj, bscheme, sizes, perm = batched_workload()
        eng.upload(btraj.unwrapped, btraj.box)
        eng.set_scheme(bscheme)
        blo = btraj.box_lo.astype(np.float32)
        bhi = (btraj.box_lo.astype(np.float64) + btraj.box.astype(np.float64)).astype(np.float32)
        eng.boxify(blo, bhi)
        bh = eng.bins_create((4, 4, 4), blo, bhi)
        for _ in range(args.warmup):
            eng.disp_bins(0, bh, 64, d4=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            eng.disp_bins(0, bh, 64, d4=False)
        result["bins_only"] = dict(call_ms=1e3 * (time.perf_counter() - t0) / max(args.steps, 1))
        eng.bins_free(bh)

    if args.only in ("", "batched"):
        btraj, bscheme, sizes, perm = batched_workload()
        shells = reference_shells([10, 20, 40, 60, 80])
        L = 61.9
        eng.upload(btraj.unwrapped[:, perm], btraj.box)   # list-nested order: lists are prefixes
        eng.set_scheme(bscheme)
        nested = [eng.list(np.arange(n, dtype=np.int32)) for n in sizes]
        G = eng.n_timegaps
        npairs = int(E.scheme_counts(eng.scheme)[2])
        units = float(sizes.sum()) * npairs
        frames_used = btraj.n_frames

        def time_plan(plan, reps):
            plan.run()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                plan.run()
            e1.record(stream)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / reps

        t0 = time.perf_counter()
        p_msd = eng.plan(nested, flags=E.PLAN_AUTOTUNE | E.PLAN_GRAPH)
        p_fs = eng.plan(nested, shells=shells, period=L, flags=E.PLAN_AUTOTUNE | E.PLAN_GRAPH)
        tune_s = time.perf_counter() - t0
        l0 = eng.launch_count()
        ms_msd = max_over_ranks(pg, time_plan(p_msd, 20))
        ms_fs = max_over_ranks(pg, time_plan(p_fs, max(2, args.steps)))
        blaunch = eng.launch_count() - l0
        info_msd, info_fs = p_msd.info(), p_fs.info()
        share = p_msd.sharing()
        p_msd.close()
        p_fs.close()
        # the same lists without work sharing (one unit of work per list)
        ns_flags = E.PLAN_AUTOTUNE | E.PLAN_GRAPH | E.PLAN_NO_SHARING
        p_ns = eng.plan(nested, flags=ns_flags)
        ms_msd_ns = max_over_ranks(pg, time_plan(p_ns, 10))
        p_ns.close()
        p_fs_ns = eng.plan(nested, shells=shells, period=L, flags=ns_flags)
        ms_fs_ns = max_over_ranks(pg, time_plan(p_fs_ns, 1))
        p_fs_ns.close()
        # the same MSD + NGP plans through the bulk-copy-staged kernel (frames
        # streamed into a shared-memory ring by cp.async.bulk)
        os.environ["AMDAT_DISP_KERNEL"] = "bulk"
        try:
            p_bk = eng.plan(nested, flags=E.PLAN_AUTOTUNE | E.PLAN_GRAPH)
            p_bk_ns = eng.plan(nested, flags=ns_flags)
        finally:
            del os.environ["AMDAT_DISP_KERNEL"]
        ms_bulk = max_over_ranks(pg, time_plan(p_bk, 10))
        ms_bulk_ns = max_over_ranks(pg, time_plan(p_bk_ns, 10))
        p_bk.close()
        p_bk_ns.close()
        # gathered layout (original atom order, index lists) for comparison
        eng.upload(btraj.unwrapped, btraj.box)
        eng.set_scheme(bscheme)
        gathered = [eng.list(np.sort(perm[:n]).astype(np.int32)) for n in sizes]
        p_g = eng.plan(gathered, flags=E.PLAN_GRAPH)
        ms_g = max_over_ranks(pg, time_plan(p_g, 10))
        p_g.close()
        # spatial bins over the same walk (create_bin_list all 4 4 4): the MSD, and
        # MSD + F_s, of all 64 bins in one keyed pass over the 200000 atoms, with
        # membership at t0 and with persistence (t0 and t1)
        blo = btraj.box_lo.astype(np.float32)
        bhi = (btraj.box_lo.astype(np.float64) + btraj.box.astype(np.float64)).astype(np.float32)
        eng.boxify(blo, bhi)
        bh = eng.bins_create((4, 4, 4), blo, bhi)
        bin_ms = {}
        for tag, kw in (("msd", {"d4": False}), ("msd_ngp", {}), ("msd_persistent", {"persistent": 1, "d4": False}),
                        ("msd_fs", {"shells": shells, "period": L, "d4": False})):
            eng.disp_bins(0, bh, 64, **kw)  # warm-up
            torch.cuda.synchronize()
            eng.profile_reset(True)
            t0 = time.perf_counter()
            reps = 5
            for _ in range(reps):
                out_b = eng.disp_bins(0, bh, 64, **kw)
            wall = (time.perf_counter() - t0) / reps
            nk, kms = eng.profile_kernel("disp_bins_kernel")
            eng.profile_reset(False)
            bin_ms[tag] = dict(kernel_ms=max_over_ranks(pg, kms / max(nk, 1)), call_ms=1e3 * wall,
                               terms=int(out_b["count"].sum()))
        eng.bins_free(bh)
        # plain FP64 path on the largest list (MSD + F_s), the mixed rate on the same list
        big = gathered[-1]
        t1 = time.perf_counter()
        eng.disp(big, shells=shells, period=L, precision=1)
        plain_rate = float(sizes[-1]) * npairs / (time.perf_counter() - t1)
        alg_bytes = float(sizes.sum()) * frames_used * 12
        unit_bytes = float(share["unit_atoms"]) * frames_used * 12
        result["batched"] = dict(
            ms_msd=ms_msd, ms_fs=ms_fs, ms_gathered=ms_g, units=units, tune_s=tune_s,
            info_msd=info_msd, info_fs=info_fs, launches=blaunch, plain_rate=plain_rate,
            alg_bytes=alg_bytes, unit_bytes=unit_bytes, share=share, ms_msd_ns=ms_msd_ns,
            ms_fs_ns=ms_fs_ns, ms_bulk=ms_bulk, ms_bulk_ns=ms_bulk_ns,
            nvec=int(shells[1][-1]), sum_n=int(sizes.sum()), npairs=npairs,
            bins=bin_ms, n_atoms=int(btraj.n_atoms), frames=int(frames_used))

    if args.only in ("", "cli") and rank == 0:
        result["cli"] = cli_bench()

    if args.only in ("", "pairs"):
        # RDF + van Hove self/distinct: N=64000, L=42.3, 50 linear frames, sigma=0.1
        from amdat_gb300 import synth
        PF = args.pair_frames
        pscheme = synth.TimeScheme.linear(PF, 1.0)
        ptraj = synth.random_walk(64000, 42.3, pscheme, 0.1, seed=3, time_scaled=False)
        eng.upload(ptraj.unwrapped, ptraj.box)
        eng.set_scheme(pscheme)
        frames = np.arange(PF, dtype=np.int32)
        eng.rdf(0, 0, frames[:2], 21.15, 500)  # warm-up
        torch.cuda.synchronize()
        eng.profile_reset(True)
        t0 = time.perf_counter()
        counts = eng.rdf(0, 0, frames, 21.15, 500)
        rdf_s = time.perf_counter() - t0
        n_rdf, ms_rdf = eng.profile_kernel("pair_hist_kernel")
        eng.profile_reset(False)
        gs_units = 64000.0 * int(E.scheme_counts(eng.scheme)[2])
        eng.disp(0, n_bins=200, bin_max=5.0)
        t0 = time.perf_counter()
        out = eng.disp(0, n_bins=200, bin_max=5.0)
        gs_s = time.perf_counter() - t0
        # distinct van Hove over every one of the 1226 time pairs of the 50-frame scheme
        npairs_gd = int(E.scheme_counts(eng.scheme)[2])
        eng.profile_reset(True)
        t0 = time.perf_counter()
        gd_counts = eng.vhd(0, 0, 5.0, 200)
        gd_s = time.perf_counter() - t0
        n_gd, ms_gd = eng.profile_kernel("pair_hist_cells_kernel")
        eng.profile_reset(False)
        # the same G_d through the all-pairs pass (every ordered pair visited)
        os.environ["AMDAT_PAIR_CELLS"] = "off"
        try:
            eng.profile_reset(True)
            t0 = time.perf_counter()
            gd_all = eng.vhd(0, 0, 5.0, 200)
            gd_all_s = time.perf_counter() - t0
            _, ms_gd_all = eng.profile_kernel("pair_hist_kernel")
            eng.profile_reset(False)
        finally:
            del os.environ["AMDAT_PAIR_CELLS"]
        gd_same = bool(np.array_equal(gd_counts, gd_all))
        n = 64000.0
        result["pairs"] = dict(frames=PF, rdf_rate=PF * n * (n - 1) / rdf_s, rdf_ms=1e3 * rdf_s,
                               rdf_kernel_ms=ms_rdf, rdf_launches=n_rdf,
                               gs_rate=gs_units / gs_s, gs_ms=1e3 * gs_s,
                               gd_rate=npairs_gd * n * (n - 1) / gd_s, gd_ms=1e3 * gd_s,
                               gd_kernel_ms=ms_gd, gd_pairs=npairs_gd, rdf_total=int(counts.sum()),
                               gd_all_ms=1e3 * gd_all_s, gd_all_kernel_ms=ms_gd_all, gd_same=gd_same,
                               gd_cells=int(math.floor(42.3 / (5.0 * (1 + 1e-4)))) ** 3)

    if args.only in ("", "structure"):
        result["structure"] = structure_bench(torch, stream, local, args)

    # CPU baseline on rank 0 (bounded samples of both workloads)
    # The same oracle runs are the parity check of the timed results: the sampled
    # rho elements of the kept step's middle frame, and the MSD and F_s sums of the
    # last timed MSD step (all outside the timed regions).
    cpu = None
    if rank == 0 and not args.no_cpu and args.only in ("", "isf", "msd"):
        from oracle import build_oracle
        build_oracle.build_lib()
        threads = os.cpu_count() or 1
        if "isf" in result:
            r = result["isf"]
            traj, _, lat = isf_workload(args.frames)
            rate, sample, dt, idx, ref = cpu_rhok_sample(traj, r["kv"], threads)
            cpu = {"value": rate, "unit": "atom·k/s", "cores": threads, "kind": "port",
                   "sample": sample + f" ({dt:.1f} s)"}
            d = (r["rho_mid"][idx].astype(np.float64) - ref[0]) / math.sqrt(traj.n_atoms)
            r["checks"]["rho_vs_fp64_oracle"] = {
                "frame": traj.n_frames // 2, "vectors": int(len(idx)),
                "rms_over_sqrtN": float(np.sqrt((d ** 2).mean())),
                "worst_over_sqrtN": float(np.abs(d).max()),
                "bound": "rms <= 1e-6, worst <= 3e-6 (times sqrt(N))"}
        if "msd" in result:
            m = result["msd"]
            mtraj, mscheme = msd_workload()
            r2, s2, dt2, d2, fs = cpu_disp_sample(mtraj, mscheme, lattice_shell(16.8, 7.0, 7.2), threads)
            m["cpu"] = {"value": r2, "unit": "atom·time-pairs/s", "cores": threads,
                        "kind": "port", "sample": s2 + f" ({dt2:.1f} s)"}
            o = m["out"]
            c = np.maximum(o["cnt"], 1)
            m["checks"] = {
                "msd_worst_rel": float((np.abs(o["sum_d2"] - d2) / np.maximum(np.abs(d2), 1e-300))[o["cnt"] > 0].max()),
                "fs_worst_abs": float(np.abs(o["fs"] / c - fs / (c * m["nvec"])).max()),
                "bound": "MSD <= 1e-6 relative, F_s <= 1e-6 absolute, against the FP64 oracle over every "
                         "time pair and atom"}

    if rank != 0:
        eng.close()
        return
    line = {"metric": METRIC, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Gaussian random walk)"}
    if "isf" in result:
        r = result["isf"]
        hbm = peaks.get("hbm_gbs")
        line.update({
            "value": r["value"], "unit": "atom·k/s", "ms_per_step": r["ms"],
            "config": {"workload": f"coherent ISF + S(k): rho_k(t) over all half-space lattice k "
                                   f"with |k|<=20 ({r['nk']} vectors, {r['ns']} shells of 0.1), "
                                   f"N={r['N']} (80:20), L=33.6, {r['T']} linear frames, "
                                   f"F(k,t) over all time pairs, S(k)",
                       "global_batch": r["N"], "frames": r["T"], "vectors": r["nk"],
                       "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (trajectory 154 MB, rho table "
                             f"{r['T'] * r['nk'] * 8 / 1e9:.1f} GB); no flush"},
            "roofline": (
                {"bound": "tensor", "achieved": r["achieved"],
                 "peak": peaks.get("bf16_tflops_sustained", 1700.0), "unit": "TFLOP/s",
                 "frac": r["achieved"] / peaks.get("bf16_tflops_sustained", 1700.0),
                 "traffic": TC_DRAM_BYTES_PER_FRAME * r["T"] * r["steps"] / max(r["n_lat"], 1),
                 "traffic_rule": "bytes per launch: ncu dram__bytes_read+write of a 2-frame "
                                 "launch per frame x frames per launch",
                 "kernel": r["kname"], "kernel_ms_per_step": r["lat_ms"],
                 "kernel_launches": r["n_lat"],
                 "flops_per_step": 8.0 * r["N"] * r["T"] * r["nk"],
                 "achieved_rule": "algorithmic: 8 flops (one complex MAC) per atom*vector",
                 "issued_tensor_tflops": r["issued"],
                 "issued_rule": "3 fp16 split passes x 8 flops x atoms x frames x tile entries "
                                "(64 complex rows x up to 128 nz per tile, incl. tile padding)",
                 "peak_source": "bf16_tflops_sustained of MEASURED_PEAKS.json (fp16 and bf16 "
                                "dense rates are equal; the kernel runs inside a seconds-long step)",
                 "fp32_pipe_peak_tflops": r["fp32_peak_max"]}
                if r["kname"] == "rhok_tc_kernel" else
                {"bound": "fp32", "achieved": r["achieved"],
                 "peak": r["fp32_peak_max"], "unit": "TFLOP/s",
                 "frac": r["achieved"] / r["fp32_peak_max"], "traffic": None,
                 "kernel": r["kname"], "kernel_ms_per_step": r["lat_ms"],
                 "kernel_launches": r["n_lat"],
                 "flops_per_step": 8.0 * r["N"] * r["T"] * r["nk"],
                 "peak_source": "FP32 FMA peak = 2 x 128 lanes x SMs x sm_max_mhz of "
                                "MEASURED_PEAKS.json (the file has no FP32 figure)",
                 "hbm_peak_gbs": hbm}),
            "e2e": {"value": r["e2e"], "unit": "atom·k/s", "h2d_bytes_per_step": r["h2d"],
                    "d2h_bytes_per_step": r["d2h"], "ms_per_step": r["e2e_ms"]},
            "gpu_launches": r["launches"],
            "clocks": r["clocks"],
            "fp64_plain": {"value": r["plain_rate"], "unit": "atom·k/s",
                           "sample": "1 frame, all vectors",
                           "mixed_over_plain": r["value"] / world / r["plain_rate"]},
            "isf_correlator_ms": r["isf_ms"],
            "parity": r["checks"],
        })
    if cpu:
        line["cpu_baseline"] = cpu
    if "msd" in result:
        m = result["msd"]
        sec = {"workload": f"MSD+NGP+F_s: N=4000, L=16.8, exponential 10x27 base 1.3, "
                           f"{m['npairs']} time pairs, F_s over {m['nvec']} lattice vectors "
                           f"|k| in [7.0,7.2]",
               "value": m["value"], "unit": "atom·time-pairs/s", "ms_per_step": m["ms"],
               "kernel_ms": m["kernel_ms"],
               "plan_graph": {"value": m["plan_value"], "ms_per_step": m["plan_ms"],
                              "note": "the same pass as a prepared plan replayed from a CUDA graph"},
               "fp64_plain": {"value": m["plain"], "mixed_over_plain": m["value"] / world / m["plain"]},
               "e2e": {"value": m["e2e"], "unit": "atom·time-pairs/s", "h2d_bytes_per_step": m["h2d"],
                       "d2h_bytes_per_step": m["d2h"], "ms_per_step": m["e2e_ms"]},
               "l2": "trajectory 13 MB < L2: a 256 MB write flushes L2 between timed steps"}
        fp32_peak = 2 * FP32_LANES_PER_SM * sm_count * float(peaks.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12
        fs_tflops = 8.0 * m["npairs"] * 4000 * m["nvec"] / (m["kernel_ms"] / 1e3) / 1e12
        sec["roofline"] = {
            "bound": "fp32", "achieved": fs_tflops, "peak": fp32_peak, "unit": "TFLOP/s",
            "frac": fs_tflops / fp32_peak, "traffic": None, "kernel": "disp_mixed_kernel",
            "kernel_ms": m["kernel_ms"],
            "achieved_rule": "algorithmic: 8 FP32 flops per atom x time pair x vector (one complex multiply "
                             "and accumulate of a recursive phase), 2246 vectors, 316 pairs, 4000 atoms",
            "peak_source": "FP32 FMA peak = 2 x 128 lanes x SMs x sm_max_mhz of MEASURED_PEAKS.json"}
        if "cpu" in m:
            sec["cpu_baseline"] = m["cpu"]
        if "checks" in m:
            sec["parity"] = m["checks"]
        if "value" not in line:
            line.update({"value": m["value"], "unit": "atom·time-pairs/s",
                         "ms_per_step": m["ms"], "config": {"workload": sec["workload"]},
                         "e2e": sec["e2e"], "roofline": sec["roofline"]})
            line["msd_detail"] = {k: v for k, v in sec.items()
                                  if k not in ("workload", "value", "unit", "ms_per_step", "e2e", "roofline")}
        else:
            line["secondary"] = sec
    if "batched" in result:
        b = result["batched"]
        hbm = peaks.get("hbm_gbs", 6699.5)
        gbs = b["unit_bytes"] / (b["ms_msd"] / 1e3) / 1e9
        gbs_ns = b["alg_bytes"] / (b["ms_msd_ns"] / 1e3) / 1e9
        line["batched"] = {
            "workload": f"64 lists (log-uniform 100..50000, nested prefixes of one permutation, "
                        f"sum N = {b['sum_n']}) of a 200000-atom walk, exponential 12x30 base 1.25, "
                        f"{b['npairs']} time pairs; one persistent launch per pass, CUDA graph, "
                        f"autotuned tiles",
            "sharing": {"units": b["share"]["n_units"], "unit_atoms": b["share"]["unit_atoms"],
                        "list_atoms": b["share"]["list_atoms"],
                        "rule": "membership classes: atoms in exactly the same lists are one unit, "
                                "processed once per time pair; list sums are sums of their classes"},
            "msd_ngp": {"value": b["units"] / (b["ms_msd"] / 1e3), "unit": "atom·time-pairs/s",
                        "ms_per_step": b["ms_msd"], "tile": b["info_msd"],
                        "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                                     "frac": gbs / hbm, "algorithmic_bytes": b["unit_bytes"],
                                     "bytes_rule": "unit atoms x 361 frames x 12 B (each shared "
                                                   "unit's trajectory once)"},
                        "per_list": {"value": b["units"] / (b["ms_msd_ns"] / 1e3),
                                     "ms_per_step": b["ms_msd_ns"],
                                     "roofline": {"bound": "hbm", "achieved": gbs_ns, "peak": hbm,
                                                  "unit": "GB/s", "frac": gbs_ns / hbm,
                                                  "algorithmic_bytes": b["alg_bytes"],
                                                  "bytes_rule": "sum_l N_l x 361 frames x 12 B "
                                                                "(each list's trajectory once)",
                                                  "unique_atom_frac": b["unit_bytes"] / (b["ms_msd_ns"] / 1e3) / 1e9 / hbm,
                                                  "unique_atom_rule": "unit atoms x 361 frames x 12 B: the floor "
                                                                      "for nested lists (every atom once)",
                                                  "dram_bytes_ncu": PERLIST_DRAM_BYTES,
                                                  "dram_frac": PERLIST_DRAM_BYTES / (b["ms_msd_ns"] / 1e3) / 1e9 / hbm,
                                                  "dram_rule": "physical DRAM bytes of one launch (one ncu "
                                                               "capture) over this launch's event time; nested "
                                                               "lists re-read frames from L2"}},
                        "gathered_layout_ms": b["ms_gathered"],
                        "bulk_staged": {"ms_per_step": b["ms_bulk"], "per_list_ms_per_step": b["ms_bulk_ns"],
                                        "frac": b["unit_bytes"] / (b["ms_bulk"] / 1e3) / 1e9 / hbm,
                                        "per_list_frac": b["alg_bytes"] / (b["ms_bulk_ns"] / 1e3) / 1e9 / hbm,
                                        "rule": "the same MSD + NGP plans through disp_bulk_kernel (each "
                                                "(pair, 512-atom) segment's six planes streamed into a "
                                                "4-stage shared-memory ring by cp.async.bulk, "
                                                "AMDAT_DISP_KERNEL=bulk); frac in the same bytes as above"}},
            "msd_ngp_fs": {"value": b["units"] / (b["ms_fs"] / 1e3), "unit": "atom·time-pairs/s",
                           "ms_per_step": b["ms_fs"], "tile": b["info_fs"],
                           "per_list": {"value": b["units"] / (b["ms_fs_ns"] / 1e3),
                                        "ms_per_step": b["ms_fs_ns"]},
                           "shells": "reference q-vector shells m=10,20,40,60,80 "
                                     f"({b['nvec']} vectors), L=61.9",
                           "fp64_plain_largest_list": b["plain_rate"],
                           "mixed_over_plain": (b["units"] / (b["ms_fs"] / 1e3)) / b["plain_rate"]},
            "autotune_s": b["tune_s"], "gpu_launches": b["launches"]}
        # binned pass: every atom in every time pair, keyed by its bin
        bunits = float(b["n_atoms"]) * b["npairs"]
        bbytes = float(b["n_atoms"]) * b["frames"] * 16.0
        bins_line = {"workload": "create_bin_list all 4 4 4 (64 bins) over the same 200000-atom walk, all "
                                 f"{b['npairs']} time pairs, one keyed pass for every bin",
                     "unit": "atom·time-pairs/s",
                     "bytes_rule": f"atoms x {b['frames']} frames x 16 B (FP32 xyz + int32 bin, each frame once)"}
        for tag, v in b["bins"].items():
            gb = bbytes / (v["kernel_ms"] / 1e3) / 1e9
            bins_line[tag] = {"value": bunits / (v["kernel_ms"] / 1e3), "kernel_ms": v["kernel_ms"],
                              "call_ms": v["call_ms"], "member_terms": v["terms"],
                              "roofline": {"bound": "hbm", "achieved": gb, "peak": hbm, "unit": "GB/s",
                                           "frac": gb / hbm}}
        # F_s per bin: one SFU cosine per member term and vector, against the MUFU rate
        v = b["bins"]["msd_fs"]
        cos_rate = v["terms"] * b["nvec"] / (v["kernel_ms"] / 1e3)
        mufu_peak = MUFU_PER_SM_CLK * sm_count * float(peaks.get("sm_max_mhz", 2070.0)) * 1e6
        bins_line["msd_fs"]["roofline"] = {
            "bound": "sfu", "achieved": cos_rate / 1e9, "peak": mufu_peak / 1e9, "unit": "G cos/s",
            "frac": cos_rate / mufu_peak,
            "rule": f"one MUFU cosine per member term x vector ({b['nvec']} vectors); peak = 16 MUFU "
                    "results per clock per SM x SMs x sm_max_mhz"}
        line["batched"]["bins"] = bins_line
        if "value" not in line:
            line.update({"value": b["units"] / (b["ms_fs"] / 1e3), "unit": "atom·time-pairs/s",
                         "ms_per_step": b["ms_fs"], "config": {"workload": line["batched"]["workload"]}})
    if "cli" in result:
        c = result["cli"]
        line["cli"] = {
            "workload": f"AMDAT input script (custom dump {c['dump_mb']:.0f} MB: {c['atoms']} atoms x "
                        f"{c['frames']} frames; msd, ngp, isfs shell 36, vhs 100 bins) through the "
                        "command-line driver, process start to exit, best of 3",
            "script_s": c["script_s"], "ingest_s": c["ingest_s"], "analyses_s": c["analyses_s"],
            "ingest_mb_per_s": c["dump_mb"] / c["ingest_s"],
            "note": "ingest = the system block alone (parse, upload, CUDA context); analyses_s = script - ingest"}
    if "pairs" in result:
        q = result["pairs"]
        fp32_peak = 2 * FP32_LANES_PER_SM * sm_count * float(peaks.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12
        n = 64000.0
        rdf_fl = 10.0 * q["frames"] * n * (n - 1) / 2 / (q["rdf_kernel_ms"] / 1e3) / 1e12
        # the cell pass visits each atom's 27 neighbour cells: ~27 / cells of the pairs
        gd_visited = q["gd_pairs"] * n * n * 27.0 / q["gd_cells"]
        gd_fl = 10.0 * gd_visited / (q["gd_kernel_ms"] / 1e3) / 1e12
        gd_all_fl = 10.0 * q["gd_pairs"] * n * (n - 1) / (q["gd_all_kernel_ms"] / 1e3) / 1e12
        pair_rule = ("algorithmic: 10 FP32 flops per visited pair (3 differences, 3 minimum-image "
                     "corrections, 3 multiply-adds of |r|^2, 1 bin division); peak = FP32 FMA peak "
                     "= 2 x 128 lanes x SMs x sm_max_mhz")
        line["pairs"] = {
            "workload": f"N=64000, L=42.3, {q['frames']} linear frames (sigma 0.1): RDF 500 bins to L/2 "
                        f"over all frames; G_s 200 bins to 5.0 and G_d 200 bins to 5.0 over all "
                        f"{q['gd_pairs']} time pairs",
            "rdf": {"value": q["rdf_rate"], "unit": "ordered pairs/s", "ms_per_step": q["rdf_ms"],
                    "kernel_ms": q["rdf_kernel_ms"], "counted_pairs_in_range": q["rdf_total"],
                    "roofline": {"bound": "fp32", "achieved": rdf_fl, "peak": fp32_peak, "unit": "TFLOP/s",
                                 "frac": rdf_fl / fp32_peak, "kernel": "pair_hist_kernel",
                                 "rule": pair_rule + "; the symmetric pass visits each unordered pair once"}},
            "vhs": {"value": q["gs_rate"], "unit": "atom·time-pairs/s", "ms_per_step": q["gs_ms"]},
            "vhd": {"value": q["gd_rate"], "unit": "ordered pairs/s", "ms_per_step": q["gd_ms"],
                    "kernel_ms": q["gd_kernel_ms"],
                    "unit_rule": "every ordered pair of every time pair (the reference's loop), per second",
                    "roofline": {"bound": "fp32", "achieved": gd_fl, "peak": fp32_peak, "unit": "TFLOP/s",
                                 "frac": gd_fl / fp32_peak, "kernel": "pair_hist_cells_kernel",
                                 "rule": pair_rule + f"; visited pairs = time pairs x N^2 x 27 / "
                                                     f"{q['gd_cells']} cells (each atom's 27 neighbour "
                                                     f"cells of width >= 5.0)"},
                    "all_pairs": {"ms_per_step": q["gd_all_ms"], "kernel_ms": q["gd_all_kernel_ms"],
                                  "counts_equal": q["gd_same"],
                                  "roofline_frac": gd_all_fl / fp32_peak,
                                  "rule": "the same call with AMDAT_PAIR_CELLS=off: every ordered pair "
                                          "visited by pair_hist_kernel"}}}
    if "perlist" in result:
        line["perlist"] = result["perlist"]
    if "bins_only" in result:
        line["bins_only"] = result["bins_only"]
    if "structure" in result:
        line["structure"] = result["structure"]
        if "value" not in line:
            st = result["structure"]
            line.update({"value": st["value"], "unit": st["unit"], "ms_per_step": st["ms_per_step"],
                         "config": {"workload": st["workload"]}, "e2e": st["e2e"],
                         "gpu_launches": st["gpu_launches"]})
    print(json.dumps(line), flush=True)
    eng.close()


if __name__ == "__main__":
    main()
