#!/usr/bin/env python
"""Throughput benchmark of the analytic Kerr ray tracer on GB300.

Workload (one "step"): the production-size FP64 drop-in case — a 512 x 512 image-plane
grid over alpha, beta in [-10, 10] M, spin a ~ U[0, 0.998) and inclination
theta_o ~ U[1, 89] deg drawn with numpy default_rng(seed = rank), observer at r_o = 1e4 M,
raytrace_ana with ngeo = 400 Mino samples per ray, plus the equatorial source radius
r_equatorial for the orders n = 0, 1, 2 on every pixel. Inputs are synthetic (the
reference has no dataset); they live in HBM before the timed region.

Metric: rays/s (whole job, all ranks). Also reported: geodesic points/s.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--case full|small]

--impl reference times the reference's own CPU algorithm for this path (the oracle port
under oracle/, numpy + scipy.special) on all host cores over a bounded seeded sample of
the same workload. --case small runs a 128 x 128 grid of the same draw (for ncu captures).
Multi-GPU: launched by torch.distributed.run, one rank per GPU; the seed-0 image's pixels
are split into N contiguous ranges, one per rank (rays are independent: no data-path
collective), so every N traces the same image (strong scaling); a barrier + CUDA synchronize
bracket the timed steps and the max time over ranks is reported.

On one GPU the default run also measures the other configurations of the target and adds
them to the same JSON line under "configurations" (--no-extras skips them): the
mixed-precision 2048^2-plus-band workload against the FP64 recurrence and the plain FP64
kernel with the error statistics, the 64-image batch, the differentiable image
(image + gradient per second) and the FP64 drop-in over the draws of seeds 0-7.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GRID = 512
LIM = 10.0
NGEO = 400
ORDERS = (0, 1, 2)
R_O = 1.0e4
CPU_SAMPLE_RAYS = 16384      # rays of the bounded CPU sample (every 16th pixel of the grid)
# FP64 floating-point work of the sample kernel (addition-theorem recurrence, chunks of 64)
# per geodesic point on this workload, from an ncu capture of one launch on the 128x128 case
# (--case small): (dadd + dmul + 2 dfma thread instructions) / points.
# Used for roofline.achieved. FP64_INST_PER_POINT: FP64 pipe instructions (dadd + dmul +
# dfma) per point, against the pipe's rate (fp64_peak / 2 instructions per second).
FP64_FLOP_PER_POINT = 545.1
FP64_INST_PER_POINT = 352.3
# DRAM bytes per point of the same capture (dram__bytes_read + dram__bytes_write) / points; the
# capture's 315 MB of output is 2.4x L2, so ~14 % of its writes are still in L2 when it ends
DRAM_BYTES_PER_POINT = 46.19
BYTES_PER_POINT = 48          # t, r, theta, phi, sigma, Mino tau written per point (8 B each)
L2_FLUSH_BYTES = 256 << 20


def shard(npix, rank, world):
    """Contiguous pixel range [lo, hi) of rank out of world (sizes differ by at most one)."""
    lo = npix * rank // world
    hi = npix * (rank + 1) // world
    return lo, hi


def workload(seed, grid=GRID):
    rng = np.random.default_rng(seed)
    a = float(rng.uniform(0, 0.998))
    th_o = float(rng.uniform(1, 89)) * np.pi / 180
    x = np.linspace(-LIM, LIM, grid)
    A, B = np.meshgrid(x, x)
    return a, th_o, A.flatten(), B.flatten()


# ---------------------------------------------------------------------------
# CPU: the reference algorithm (oracle port) on host cores
# ---------------------------------------------------------------------------

def _cpu_chunk(args):
    a, th_o, A, B, ngeo = args
    from oracle import kgeo_oracle as ko
    import warnings
    warnings.filterwarnings('ignore')
    ko.raytrace(a, R_O, th_o, A, B, ngeo)
    for m in ORDERS:
        ko.r_equatorial(a, R_O, th_o, m, A, B)
    return len(A)


def cpu_sample(seed):
    a, th_o, A, B = workload(seed)
    idx = np.arange(0, A.size, A.size // CPU_SAMPLE_RAYS)[:CPU_SAMPLE_RAYS]
    return a, th_o, A[idx], B[idx]


def _pool_warm(_):
    from oracle import kgeo_oracle  # noqa: F401  (worker start-up and imports outside every timing)
    time.sleep(0.3)
    return 0


def make_pool():
    import multiprocessing as mp
    cores = len(os.sched_getaffinity(0))
    os.environ.setdefault('OMP_NUM_THREADS', '1')
    os.environ.setdefault('OPENBLAS_NUM_THREADS', '1')
    pool = mp.get_context('spawn').Pool(cores)
    pool.map(_pool_warm, range(2 * cores), chunksize=1)
    return pool, cores


def cpu_run(pool, cores, seed):
    """One pass of the bounded sample over all cores; returns (rays, seconds)."""
    a, th_o, A, B = cpu_sample(seed)
    chunks = np.array_split(np.arange(A.size), cores * 4)
    t0 = time.perf_counter()
    n = sum(pool.map(_cpu_chunk, [(a, th_o, A[c], B[c], NGEO) for c in chunks if c.size]))
    return n, time.perf_counter() - t0


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------

class Clocks:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,'
         'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
         'clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.idx), '--query-gpu=' + self.Q,
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == 'active':
                    reasons.add(n)
        if not sm:
            return None
        return {'sm_mhz': float(np.median(sm)), 'sm_max_mhz': mx, 'reasons': sorted(reasons), 'samples': len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            return json.load(f)
    except OSError:
        return {}


def dist_env():
    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', '1'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return rank, world, local


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def run_ours(args):
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl' if torch.cuda.is_available() else 'gloo')
    from kgeo_gb300 import device as dev
    from kgeo_gb300 import equatorial_lensing as el
    from kgeo_gb300 import kerr_raytracing_ana as kra

    grid = GRID if args.case == 'full' else 128
    a, th_o, A_all, B_all = workload(0, grid)
    lo, hi = shard(A_all.size, rank, world)
    A, B = A_all[lo:hi], B_all[lo:hi]
    npix = A.size
    al, be = dev.as_device(A), dev.as_device(B)
    prep = dev.PreparedRays(a, R_O, th_o, al, be, ngeo=NGEO)
    out = prep.alloc()
    flags = torch.zeros(1, dtype=torch.int32, device=al.device)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=al.device)
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def step(rec=None):
        flush.zero_()
        e = [ev() for _ in range(4)] if rec is not None else None
        if e:
            e[0].record(stream)
        prep.setup()
        if e:
            e[1].record(stream)
        prep.samples(out, flags=flags)
        if e:
            e[2].record(stream)
        el.r_equatorial_device(a, R_O, th_o, ORDERS, al, be)
        if e:
            e[3].record(stream)
            rec.append(e)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = Clocks(local)
    clocks.start()
    recs = []
    t0 = ev()
    t1 = ev()
    t0.record(stream)
    for _ in range(args.steps):
        step(recs)
    t1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    elapsed = t0.elapsed_time(t1) / 1e3
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([elapsed], dtype=torch.float64, device=al.device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        dist.barrier()
        elapsed = float(tt.item())
    setup_ms = np.mean([r[0].elapsed_time(r[1]) for r in recs])
    samp_ms = np.mean([r[1].elapsed_time(r[2]) for r in recs])
    eq_ms = np.mean([r[2].elapsed_time(r[3]) for r in recs])
    rays = A_all.size * args.steps
    value = rays / elapsed
    points = npix * NGEO
    launches = 5 * args.steps  # setup + bucket scan + bucket scatter, samples, r_equatorial

    # end to end through the public API with host buffers: numpy in, numpy out
    e2e = None
    if args.steps > 0:
        # untimed passes: the page-locked host outputs come from torch's pinned-memory cache
        # in steady state
        for _ in range(2):
            g = kra.raytrace_ana(a=a, observer_coords=[0, R_O, th_o, 0], image_coords=[A, B], ngeo=NGEO,
                                 plotdata=False)
            rq = [el.r_equatorial(a, R_O, th_o, m, A, B) for m in ORDERS]
            del g, rq
        torch.cuda.synchronize()
        nsteps_e = max(1, min(args.steps, 5))
        step_ms = []
        t_e = time.perf_counter()
        for _ in range(nsteps_e):
            t_s = time.perf_counter()
            g = kra.raytrace_ana(a=a, observer_coords=[0, R_O, th_o, 0], image_coords=[A, B], ngeo=NGEO,
                                 plotdata=False)
            rq = [el.r_equatorial(a, R_O, th_o, m, A, B) for m in ORDERS]
            del g, rq
            step_ms.append((time.perf_counter() - t_s) * 1e3)
        dt = (time.perf_counter() - t_e) / nsteps_e
        if world > 1:
            import torch.distributed as dist
            tt = torch.tensor([dt], dtype=torch.float64, device=al.device)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            dt = float(tt.item())
        h2d = 2 * A_all.size * 8 * (1 + len(ORDERS))
        d2h = 6 * A_all.size * NGEO * 8 + len(ORDERS) * 4 * A_all.size * 8
        e2e = {'value': A_all.size / dt, 'unit': 'rays/s', 'h2d_bytes_per_step': h2d, 'd2h_bytes_per_step': d2h,
               'ms_per_step': dt * 1e3, 'step_ms': [round(x, 2) for x in step_ms],
               'path': 'kgeo_gb300.kerr_raytracing_ana.raytrace_ana + equatorial_lensing.r_equatorial (numpy in/out)'}

    if rank != 0:
        return
    pk = peaks()
    fp64_peak = dev.fp64_peak_tflops()
    roof = {'bound': 'fp64', 'unit': 'TFLOP/s', 'peak': fp64_peak,
            'peak_source': 'FP64 FMA loop measured live by bench.py (kgeo_measure_fp64_peak)',
            'kernel': 'stepped_kernel', 'launch_ms': samp_ms, 'points_per_launch': points,
            'traffic': DRAM_BYTES_PER_POINT * points,
            'traffic_source': 'ncu dram__bytes_read+write of a 128x128 capture, scaled by points'}
    if FP64_FLOP_PER_POINT:
        ach = FP64_FLOP_PER_POINT * points / (samp_ms * 1e-3) / 1e12
        roof.update({'achieved': ach, 'frac': ach / fp64_peak, 'fp64_flop_per_point': FP64_FLOP_PER_POINT,
                     'fp64_pipe_frac': FP64_INST_PER_POINT * points / (samp_ms * 1e-3) / (fp64_peak * 1e12 / 2)})
    else:
        roof.update({'achieved': None, 'frac': None})
    hbm = BYTES_PER_POINT * points / (samp_ms * 1e-3) / 1e9
    roof['hbm_write'] = {'achieved_gbs': hbm, 'peak_gbs': pk.get('hbm_gbs'),
                         'frac': (hbm / pk['hbm_gbs']) if pk.get('hbm_gbs') else None,
                         'bytes_per_point': BYTES_PER_POINT}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # spawned workers (no CUDA state inherited), started after the GPU timings so that no
        # worker start-up overlaps them
        pool, cores = make_pool()
        cpu_run(pool, cores, rank)  # warm the workers (imports)
        n, dt = cpu_run(pool, cores, rank)
        pool.close()
        cpu = {'value': n / dt, 'unit': 'rays/s', 'cores': cores, 'kind': 'port',
               'sample': '%d rays (every %dth pixel of the same grid and draw), ngeo=%d, r_equatorial n=0..2; '
                         'oracle/kgeo_oracle.py (numpy+scipy restatement of the reference) on a %d-process pool, '
                         '%.1f s wall' % (n, npix // CPU_SAMPLE_RAYS, NGEO, cores, dt)}
    extras = None
    if world == 1 and args.case == 'full' and not args.no_extras:
        del prep, out, flush
        torch.cuda.empty_cache()
        extras = configuration_extras(args)
    line = {
        'metric': 'Kerr rays/s: FP64 raytrace_ana (ngeo=400) + r_equatorial n=0..2, 512x512 image',
        'value': value, 'unit': 'rays/s', 'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': elapsed / args.steps * 1e3, 'higher_is_better': True, 'scaling': 'strong',
        'vs_baseline': None, 'dtype': 'f64',
        'data': 'synthetic: uniform image-plane grid, a and theta_o drawn from default_rng(0); with N ranks each '
                'traces a contiguous 1/N of the pixels',
        'config': {'workload': 'FP64 drop-in at production size (512x512 over [-10,10] M, a~U[0,0.998), '
                               'theta_o~U[1,89] deg, r_o=1e4, ngeo=400, r_equatorial n=0,1,2)',
                   'npix': npix, 'ngeo': NGEO, 'a': a, 'th_o_deg': th_o * 180 / np.pi, 'orders': list(ORDERS),
                   'precision': 'fp64', 'case': args.case,
                   'l2': 'flushed between steps (256 MiB memset); outputs 5 GB per step'},
        'points_per_s': value * NGEO, 'kernel_ms': {'ray_setup': setup_ms, 'samples': samp_ms,
                                                    'r_equatorial': eq_ms},
        'roofline': roof, 'cpu_baseline': cpu, 'e2e': e2e, 'gpu_launches': launches, 'clocks': ck,
        'configurations': extras,
    }
    print(json.dumps(line))


def configuration_extras(args):
    """The target's other configurations, measured in the same run (one GPU)."""
    import copy
    import torch
    sub = copy.copy(args)
    sub.no_cpu_baseline = True
    out = {}

    def free():
        import gc
        gc.collect()
        torch.cuda.empty_cache()

    def err_summary(e):
        if e is None:
            return None
        keep = ('max', 'rms', 'frac_above_1e-6', 'max_over_bar', 'horizon_sample_max')
        res = {k: {q: v[q] for q in keep if q in v} for k, v in e.items()
               if isinstance(v, dict) and k != 'max_over_parity_bar'}
        for k in ('max_over_parity_bar', 'parity_bar'):
            if k in e:
                res[k] = e[k]
        return res
    # configuration 3: mixed vs the FP64 recurrence and the plain FP64 kernel; both GPU paths
    # against the oracle on a seeded 1/64 subsample of the rays (band included), on the host
    # cores after the GPU timings
    sub.case, sub.steps, sub.warmup = 'mixed', 2, 3
    sub.no_cpu_baseline = False
    m = run_mixed(sub, emit=False)
    sub.no_cpu_baseline = True
    out['config3_mixed'] = {
        'rays_per_s': m['value'], 'ms_per_step': m['ms_per_step'],
        'fp64_recurrence_rays_per_s': m['fp64_recurrence']['value'], 'fp64_plain_rays_per_s': m['fp64_plain']['value'],
        'speedup_vs_fp64_recurrence': m['speedup_vs_fp64_recurrence'], 'speedup_vs_fp64_plain': m['speedup_vs_fp64_plain'],
        'mixed_vs_fp64_recurrence_error': err_summary(m['mixed_vs_fp64_error']),
        'fp64_vs_oracle_error': err_summary(m['fp64_vs_oracle_error']),
        'mixed_vs_oracle_error': err_summary(m['mixed_vs_oracle_error']),
        'oracle_rays': (m['fp64_vs_oracle_error'] or {}).get('rays'),
        'error_scales': m['error_scales'], 'clocks': m['clocks'], 'workload': m['config']['workload']}
    free()
    # configuration 4: 64 images in one persistent launch / CUDA graph
    sub.case, sub.steps, sub.warmup = 'batch', 2, 3
    b = run_batch(sub, emit=False)
    out['config4_batch'] = {
        'rays_per_s': b['value'], 'ms_per_step': b['ms_per_step'],
        'fp64_batched_recurrence_rays_per_s': b['fp64_batched_recurrence']['value'],
        'fp64_plain_rays_per_s': b['fp64_plain']['value'], 'speedup_vs_fp64_plain': b['speedup_vs_fp64_plain'],
        'speedup_vs_fp64_recurrence': b['speedup_vs_fp64_recurrence'],
        'mixed_vs_fp64_error': b['mixed_vs_fp64_error'], 'tuned': b['config']['tuned'], 'clocks': b['clocks']}
    free()
    # configuration 5: image + adjoint gradient
    sub.case, sub.steps, sub.warmup = 'image', 10, 3
    im = run_image(sub, emit=False)
    out['config5_image_grad'] = {
        'image_grad_per_s': im['value'], 'ms_per_step': im['ms_per_step'], 'kernel_ms': im['kernel_ms'],
        'e2e_image_grad_per_s': im['e2e']['value'], 'roofline_frac': im['roofline']['frac'], 'clocks': im['clocks']}
    free()
    # configuration 2 over the draws of seeds 0-7 (device rays/s of setup + samples + r_equatorial)
    from kgeo_gb300 import device as dev
    from kgeo_gb300 import equatorial_lensing as el
    stream = torch.cuda.current_stream()
    rates, draws = [], []
    for seed in range(8):
        a, th_o, A, B = workload(seed)
        al, be = dev.as_device(A), dev.as_device(B)
        prep = dev.PreparedRays(a, R_O, th_o, al, be, ngeo=NGEO)
        o = prep.alloc()

        def step():
            prep.setup()
            prep.samples(o)
            el.r_equatorial_device(a, R_O, th_o, ORDERS, al, be)
        step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(2):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        rates.append(2 * A.size / (e0.elapsed_time(e1) / 1e3))
        draws.append((round(a, 4), round(th_o * 180 / np.pi, 2)))
        del prep, o
    free()
    out['config2_seeds_0_7'] = {'rays_per_s': rates, 'min': min(rates), 'mean': float(np.mean(rates)),
                                'draws_a_thdeg': draws}
    return out


# ---------------------------------------------------------------------------
# reference arm: the reference algorithm on the host cores
# ---------------------------------------------------------------------------

def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    pool, cores = make_pool()
    a, th_o, A, B = cpu_sample(0)
    for _ in range(args.warmup):
        cpu_run(pool, cores, 0)
    tot_n, tot_t = 0, 0.0
    for _ in range(args.steps):
        n, dt = cpu_run(pool, cores, 0)
        tot_n += n
        tot_t += dt
    pool.close()
    value = tot_n / tot_t
    line = {
        'impl': 'reference',
        'metric': 'Kerr rays/s: FP64 raytrace_ana (ngeo=400) + r_equatorial n=0..2, 512x512 image',
        'value': value, 'unit': 'rays/s', 'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': tot_t / max(args.steps, 1) * 1e3, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic: uniform image-plane grid, seeded a and theta_o',
        'config': {'workload': 'FP64 drop-in at production size (512x512 over [-10,10] M, a~U[0,0.998), '
                               'theta_o~U[1,89] deg, r_o=1e4, ngeo=400, r_equatorial n=0,1,2)',
                   'npix': GRID * GRID, 'ngeo': NGEO, 'precision': 'fp64'},
        'cpu_baseline': {'value': value, 'unit': 'rays/s', 'cores': cores, 'kind': 'port',
                         'sample': 'each step: %d rays (every 16th pixel) of the seed-0 draw, ngeo=%d, '
                                   'r_equatorial n=0..2, oracle/kgeo_oracle.py on %d processes'
                                   % (A.size, NGEO, cores)},
        'e2e': {'value': value, 'unit': 'rays/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# configuration 3: mixed precision (2048^2 grid + polar band near the critical curve)
# ---------------------------------------------------------------------------

def mixed_workload(small=False):
    from kgeo_gb300.equatorial_lensing import critical_band
    a, th_o = 0.94, 17 * np.pi / 180
    # the small (ncu capture) case: 384^2 + 512 x 32 band rays, about four waves of the kernel
    n = 384 if small else 2048
    x = np.linspace(-LIM, LIM, n)
    A, B = (v.flatten() for v in np.meshgrid(x, x))
    bA, bB = critical_band(a, th_o, n_angles=512 if small else 4096, n_radii=32 if small else 256)
    return a, th_o, np.concatenate([A, bA]), np.concatenate([B, bB]), A.size


def _oracle_chunk(args):
    a, th_o, A, B, ngeo = args
    from oracle import kgeo_oracle as ko
    import warnings
    warnings.filterwarnings('ignore')
    out = ko.raytrace(a, R_O, th_o, A, B, ngeo)
    rho = ko.pole_distance(a, R_O, th_o, A, B, out['mino_times'])
    return np.stack([out['r'], out['th'], out['ph'], out['t'], out['affine_times']]), out['rclass'], rho


def error_stats(got, ref, rclass, torch, rho=None):
    """Per output max / RMS relative error with the parity scales; the horizon-adjacent last
    sample of rclass 2-4 rays is reported separately."""
    res = {}
    G = ref['r'].shape[0]
    horizon = torch.isin(rclass, torch.tensor([2, 3, 4], device=rclass.device))
    for k, scale in (('r', None), ('th', 1.0), ('ph', 1.0), ('t', R_O), ('sig', R_O)):
        x, y = got[k], ref[k]
        den = y.abs() if scale is None else torch.clamp(y.abs(), min=scale)
        e = (x - y).abs() / den
        fin = torch.isfinite(e)
        e = torch.where(fin, e, torch.zeros_like(e))
        body = e[:G - 1]
        last = e[G - 1][horizon]
        e_rest = e[G - 1][~horizon]
        mx = max(float(body.max()), float(e_rest.max()) if e_rest.numel() else 0.0)
        rms = float(torch.sqrt((body.double() ** 2).mean()))
        res[k] = {'max': mx, 'rms': rms, 'horizon_sample_max': float(last.max()) if last.numel() else 0.0,
                  'frac_above_1e-6': float((body > 1e-6).double().mean()),
                  'nonfinite_mismatch': int((torch.isfinite(x) != torch.isfinite(y)).sum())}
        if rho is not None:
            # the FP64 parity rule near elliptic-Pi poles: bar max(1e-6, 10 eps / rho) per sample
            bar = torch.clamp(10 * 2.220446049250313e-16 / rho[:G - 1], min=1e-6)
            res[k]['max_over_bar'] = float((body / bar).max())
    return res


def run_mixed(args, emit=True):
    small = args.case == 'mixed-small'
    pool = cores = None
    import torch
    from kgeo_gb300 import device as dev
    a, th_o, A, B, ngrid = mixed_workload(small)
    npix = A.size
    G = 256
    al, be = dev.as_device(A), dev.as_device(B)
    prep = dev.PreparedRays(a, R_O, th_o, al, be, ngeo=G)
    out_m = prep.alloc()
    out_d = prep.alloc()
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def timed(fn, steps, warm):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        e0, e1 = ev(), ev()
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / steps

    def step_mixed():
        prep.setup()
        prep.samples(out_m, mixed=True)

    def step_fp64():
        prep.setup()
        prep.samples(out_d)

    def step_plain():
        prep.setup()
        prep.samples(out_d, chunk=0)

    clocks = Clocks(0)
    clocks.start()
    t_mixed = timed(step_mixed, args.steps, args.warmup)
    ck = clocks.stop()
    t_plain = timed(step_plain, 1, 0)
    t_fp64 = timed(step_fp64, max(1, args.steps // 2), 1)
    errs = error_stats(out_m, out_d, prep.rclass, torch)
    # FP64 kernel against the oracle on a seeded 1/64 subsample of the same rays
    orc = orc_m = None
    if not args.no_cpu_baseline:
        pool, cores = make_pool()  # spawned after the GPU timings
        rng = np.random.default_rng(0)
        sub = np.sort(rng.choice(npix, npix // 64, replace=False))
        chunks = np.array_split(sub, cores * 4)
        parts = pool.map(_oracle_chunk, [(a, th_o, A[c], B[c], G) for c in chunks if c.size])
        pool.close()
        ref = np.concatenate([p_[0] for p_ in parts], axis=2)
        rc = np.concatenate([p_[1] for p_ in parts])
        rho = torch.from_numpy(np.concatenate([p_[2] for p_ in parts], axis=1)).to(al.device)
        idx = torch.from_numpy(sub).to(al.device)
        refd = {k: torch.from_numpy(ref[i]).to(al.device) for i, k in enumerate(('r', 'th', 'ph', 't', 'sig'))}
        rct = torch.from_numpy(rc).to(al.device)
        orc = error_stats({k: out_d[k][:, idx] for k in refd}, refd, rct, torch, rho)
        orc['rays'] = int(sub.size)
        orc_m = error_stats({k: out_m[k][:, idx] for k in refd}, refd, rct, torch, rho)
        orc_m['rays'] = int(sub.size)
        # the parity bars themselves: FP64 max(1e-10, 10 eps / rho, 10 S) and mixed
        # max(1e-6, 10 eps / rho, 10 S), S = the oracle's change under a one-ulp change of
        # lambda or eta (evaluated for the rays above the other bars); max of error / bar
        from oracle.parity import lambda_eta_sensitivity, parity_ratios
        refn = {k: ref[i] for i, k in enumerate(('r', 'th', 'ph', 't', 'sig'))}
        rho_np = rho.cpu().numpy()
        sens = lambda_eta_sensitivity(a, R_O, th_o, A[sub], B[sub], ngeo=G)
        for err, outp, tol in ((orc, out_d, 1e-10), (orc_m, out_m, 1e-6)):
            ratio = parity_ratios({k: outp[k][:, idx].cpu().numpy() for k in refn}, refn, R_O, tol, rho_np, sens)
            err['max_over_parity_bar'] = {k: float(v.max()) / tol for k, v in ratio.items()}
            err['parity_bar'] = 'max(%g, 10 eps / rho, 10 S)' % tol
            del ratio
    points = npix * G
    line = {
        'metric': 'Kerr rays/s: mixed-precision raytrace (ngeo=256), 2048^2 grid + 256x4096 critical-curve band',
        'value': npix / t_mixed, 'unit': 'rays/s', 'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': t_mixed * 1e3, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f32+f64', 'data': 'synthetic: uniform grid + polar band from critical_curve(0.94, 17 deg)',
        'config': {'workload': 'configuration 3: a=0.94, theta_o=17 deg, r_o=1e4, ngeo=256, '
                               '%d grid + %d band rays' % (ngrid, npix - ngrid), 'npix': npix, 'ngeo': G,
                   'precision': 'mixed', 'case': args.case},
        'points_per_s': points / t_mixed,
        'fp64_recurrence': {'value': npix / t_fp64, 'ms_per_step': t_fp64 * 1e3},
        'fp64_plain': {'value': npix / t_plain, 'ms_per_step': t_plain * 1e3},
        'speedup_vs_fp64_recurrence': t_fp64 / t_mixed, 'speedup_vs_fp64_plain': t_plain / t_mixed,
        'mixed_vs_fp64_error': errs, 'fp64_vs_oracle_error': orc, 'mixed_vs_oracle_error': orc_m,
        'error_scales': 'relative; floor 1 rad for theta, phi; r_o for t, sigma; max_over_bar = max of error / '
                        'max(1e-6, 10 eps / rho), rho = distance to the nearest elliptic-Pi pole',
        'clocks': ck,
        'gpu_launches': 4 * args.steps,
    }
    if emit:
        print(json.dumps(line))
    return line


# ---------------------------------------------------------------------------
# configuration 5: differentiable equatorial image (image + gradient per step)
# ---------------------------------------------------------------------------

IMG_GRID = 512
IMG_LIM = 8.0
IMG_PHYS = (0.5, 60 * np.pi / 180, 2.0, 0.8, 0.5)   # a, theta_o, p, xi, beta_r
IMG_MBAR = 2
# FP64 FLOP per pixel of the adjoint kernel on this workload (all three orders), from the
# ncu capture of one launch on the 128x128 case (--case image-small): (dadd + dmul + 2 dfma
# thread instructions) / pixels. Used for roofline.achieved.
ADJ_FLOP_PER_PIXEL = 30083
CPU_IMG_SAMPLE = 65536       # pixels of the bounded CPU sample (every 4th pixel)


def image_workload(grid=IMG_GRID):
    x = np.linspace(-IMG_LIM, IMG_LIM, grid)
    A, B = np.meshgrid(x, x)
    eps = np.random.default_rng(0).choice([-1.0, 1.0], size=5)
    return A.flatten(), B.flatten(), np.array(IMG_PHYS), np.array(IMG_PHYS) * (1 + 0.02 * eps)


def _cpu_image_chunk(args):
    """Oracle image at the parameters and at +-1e-6 in each of the five (the central
    differences a CPU user of the reference computes for the gradient), and the loss."""
    A, B, phys, tgt = args
    from oracle import kgeo_oracle as ko
    import warnings
    warnings.filterwarnings('ignore')

    def img(ph):
        return ko.make_image_px(float(ph[0]), R_O, float(ph[1]), IMG_MBAR, A, B,
                                emis=('bpl', {'p1': -ph[2], 'p2': 0.0}),
                                vel=('general', {'fac_subkep': ph[3], 'beta_r': ph[4]}))['I']
    target = img(tgt)
    L = ((img(phys) - target) ** 2).sum()
    for k in range(5):
        for sgn in (1, -1):
            q = phys.copy()
            q[k] += sgn * 1e-6
            ((img(q) - target) ** 2).sum()
    return L


def cpu_image_run(pool, cores):
    A, B, phys, tgt = image_workload()
    idx = np.arange(0, A.size, A.size // CPU_IMG_SAMPLE)[:CPU_IMG_SAMPLE]
    chunks = np.array_split(idx, cores * 2)
    t0 = time.time()
    pool.map(_cpu_image_chunk, [(A[c], B[c], phys, tgt) for c in chunks])
    dt = time.time() - t0
    return {'value': (idx.size / A.size) / dt, 'unit': 'image+grad/s', 'cores': cores, 'kind': 'port',
            'sample': '%d pixels (every %dth of the 512x512 image), 3 orders, image + 10 central-difference '
                      'images + target; oracle/kgeo_oracle.py on a %d-process pool, %.1f s wall, scaled to the '
                      'full image' % (idx.size, A.size // CPU_IMG_SAMPLE, cores, dt)}


def run_image(args, emit=True):
    small = args.case == 'image-small'
    pool = cores = None
    import torch
    from kgeo_gb300.image_grad import config_params, equatorial_image
    grid = 128 if small else IMG_GRID
    A, B, phys, tgt = image_workload(grid)
    npix = A.size
    al = torch.from_numpy(A).cuda()
    be = torch.from_numpy(B).cuda()
    with torch.no_grad():
        target = equatorial_image(config_params(*tgt), al, be, mbar_max=IMG_MBAR)
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def step(al_, be_):
        xs = [torch.tensor(v, dtype=torch.float64, requires_grad=True) for v in phys]
        I = equatorial_image(config_params(*xs), al_, be_, mbar_max=IMG_MBAR)
        L = ((I - target) ** 2).sum()
        L.backward()
        return L, xs

    for _ in range(args.warmup):
        step(al, be)
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    e0, e1 = ev(), ev()
    e0.record(stream)
    for _ in range(args.steps):
        L, xs = step(al, be)
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    t_step = e0.elapsed_time(e1) / 1e3 / args.steps
    grad = [float(x.grad) for x in xs]
    # per-kernel times on the launching stream
    from kgeo_gb300.equatorial_images import emission_model, image_adjoint_device, image_device
    from kgeo_gb300.emissivities import Emissivity
    from kgeo_gb300.velocities import Velocity
    model = emission_model(Emissivity('bpl', p1=-phys[2], p2=0.0),
                           Velocity('general', fac_subkep=phys[3], beta_r=phys[4]))
    gI = torch.ones((npix, IMG_MBAR + 1), dtype=torch.float64, device=al.device)

    def kt(fn, n=5):
        fn()
        torch.cuda.synchronize()
        a0, a1 = ev(), ev()
        a0.record(stream)
        for _ in range(n):
            fn()
        a1.record(stream)
        torch.cuda.synchronize()
        return a0.elapsed_time(a1) / 1e3 / n
    t_fwd = kt(lambda: image_device(phys[0], R_O, phys[1], 0, IMG_MBAR + 1, al, be, model))
    t_adj = kt(lambda: image_adjoint_device(phys[0], R_O, phys[1], 0, IMG_MBAR + 1, al, be, model, gI))
    # end to end: host pixel arrays in, loss and gradient out, through the public API
    Ah = torch.from_numpy(A).pin_memory()
    Bh = torch.from_numpy(B).pin_memory()
    for _ in range(2):
        step(Ah.cuda(non_blocking=True), Bh.cuda(non_blocking=True))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        L, xs = step(Ah.cuda(non_blocking=True), Bh.cuda(non_blocking=True))
        out = (float(L.detach()), [float(x.grad) for x in xs])
    t_e2e = (time.perf_counter() - t0) / args.steps
    pk = peaks()
    fp64_peak = None
    try:
        from kgeo_gb300 import device as dev
        fp64_peak = dev.fp64_peak_tflops()
    except Exception:
        pass
    roof = {'bound': 'fp64', 'unit': 'TFLOP/s', 'kernel': 'image_adjoint_kernel', 'launch_ms': t_adj * 1e3,
            'peak': fp64_peak, 'peak_source': 'FP64 FMA loop measured live by bench.py (kgeo_measure_fp64_peak)',
            'achieved': None, 'frac': None, 'fp64_flop_per_pixel': ADJ_FLOP_PER_PIXEL,
            # ncu dram__bytes_read + write of the 128x128 capture scaled by pixels (inputs and
            # grad_I are read once; the per-block partial sums are the only writes)
            'traffic': (3.674e6 + 4.1e3) * npix / 16384}
    if ADJ_FLOP_PER_PIXEL and fp64_peak:
        roof['achieved'] = ADJ_FLOP_PER_PIXEL * npix / t_adj / 1e12
        roof['frac'] = roof['achieved'] / fp64_peak
    cpu = None
    if not args.no_cpu_baseline:
        pool, cores = make_pool()  # spawned after the GPU timings
        cpu = cpu_image_run(pool, cores)
        pool.close()
    line = {
        'metric': 'image+grad/s: configuration-5 equatorial image (512x512, n=0..2) + adjoint gradient wrt '
                  '(a, theta_o, p, xi, beta_r)',
        'value': 1.0 / t_step, 'unit': 'image+grad/s', 'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': t_step * 1e3, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f64', 'data': 'synthetic: uniform image-plane grid; target image at parameters x (1 + 0.02 eps), '
                                'eps = +-1 from default_rng(0)',
        'config': {'workload': 'configuration 5: a=0.5, theta_o=60 deg, r_o=1e4, %dx%d over [-8, 8] M, orders '
                               '0..2, bpl j ~ r^-2, general velocity xi=0.8 beta_r=0.5' % (grid, grid),
                   'npix': npix, 'orders': IMG_MBAR + 1, 'case': args.case,
                   'l2': 'inputs 4 MB (compute-bound kernels; not flushed)'},
        'loss': out[0], 'grad': out[1], 'pixels_per_s': npix / t_step,
        'kernel_ms': {'image': t_fwd * 1e3, 'image_adjoint': t_adj * 1e3},
        'roofline': roof, 'cpu_baseline': cpu,
        'e2e': {'value': 1.0 / t_e2e, 'unit': 'image+grad/s', 'h2d_bytes_per_step': 2 * 8 * npix,
                'd2h_bytes_per_step': 8 * 6, 'ms_per_step': t_e2e * 1e3,
                'path': 'kgeo_gb300.image_grad.equatorial_image (torch.autograd.Function) from pinned host arrays'},
        'gpu_launches': 3 * args.steps, 'clocks': ck,
    }
    if emit:
        print(json.dumps(line))
    return line


# ---------------------------------------------------------------------------
# polarised image: the reference's tests/test_images.py configuration at full size
# ---------------------------------------------------------------------------

POL_NX = 800
POL_MBAR = 2
POL_MODEL = dict(a=0.7, inc=45.0, fac_subkep=0.6, beta_phi=0.8, beta_r=0.7)
# FP64 FLOP per pixel of the polarised image kernel (three orders), from an ncu capture of one
# launch (--case polimage-small): (dadd + dmul + 2 dfma thread instructions) / pixels, and the
# FP64 pipe instructions (dadd + dmul + dfma) per pixel.
POL_FLOP_PER_PIXEL = 10445
POL_FP64_INST_PER_PIXEL = 6800
CPU_POL_SAMPLE = 160000


def pol_workload(nx=POL_NX):
    psize = 20. / nx
    side = np.linspace(-10., -10. + nx * psize, nx)   # make_image's grid
    A, B = np.meshgrid(side, side)
    return A.flatten(), B.flatten()


def _pol_objects():
    from kgeo_gb300.bfields import Bfield
    from kgeo_gb300.emissivities import Emissivity
    from kgeo_gb300.velocities import Velocity
    m = POL_MODEL
    return (Emissivity('ring'), Velocity('general', fac_subkep=m['fac_subkep'], beta_phi=m['beta_phi'],
                                         beta_r=m['beta_r']), Bfield('bz_guess', C=1.))


def _cpu_pol_chunk(args):
    A, B = args
    from oracle import kgeo_oracle as ko
    import warnings
    warnings.filterwarnings('ignore')
    m = POL_MODEL
    ko.make_image_px(m['a'], np.inf, m['inc'] * np.pi / 180, POL_MBAR, A, B, emis=('ring', {}),
                     vel=('general', {'fac_subkep': m['fac_subkep'], 'beta_phi': m['beta_phi'],
                                      'beta_r': m['beta_r']}),
                     specind=1., bfield=('bz_guess', {'C': 1.}), polarization=True)
    return len(A)


def run_polimage(args):
    small = args.case == 'polimage-small'
    pool = cores = None
    import torch
    from kgeo_gb300.equatorial_images import emission_model, image_device, image_options, make_image
    nx = 160 if small else POL_NX
    A, B = pol_workload(nx)
    npix = A.size
    norders = POL_MBAR + 1
    m = POL_MODEL
    th_o = m['inc'] * np.pi / 180
    em, ve, bf = _pol_objects()
    model = emission_model(em, ve, 1.)
    opts = image_options(bf, polarization=True)
    al = torch.from_numpy(A).cuda()
    be = torch.from_numpy(B).cuda()
    outs = ('I', 'Q', 'U', 'g', 'r_s', 'Ir', 'sinthb', 'nmax', 'npol')
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    for _ in range(args.warmup):
        image_device(m['a'], np.inf, th_o, 0, norders, al, be, model, outputs=outs, options=opts)
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    e0, e1 = ev(), ev()
    e0.record(stream)
    for _ in range(args.steps):
        image_device(m['a'], np.inf, th_o, 0, norders, al, be, model, outputs=outs, options=opts)
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    t_step = e0.elapsed_time(e1) / 1e3 / args.steps
    # end to end through the drop-in make_image: host grid in, nine host arrays out
    for _ in range(2):
        make_image(m['a'], np.inf, th_o, POL_MBAR, -10., 10., -10., 10., 20. / nx, emissivity=em, velocity=ve,
                   bfield=bf, polarization=True, specind=1.)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        res = make_image(m['a'], np.inf, th_o, POL_MBAR, -10., 10., -10., 10., 20. / nx, emissivity=em,
                         velocity=ve, bfield=bf, polarization=True, specind=1.)
    t_e2e = (time.perf_counter() - t0) / args.steps
    lit = float((res[0] > 0).mean())
    fp64_peak = None
    try:
        from kgeo_gb300 import device as dev
        fp64_peak = dev.fp64_peak_tflops()
    except Exception:
        pass
    roof = {'bound': 'fp64', 'unit': 'TFLOP/s', 'kernel': 'image_kernel<true>', 'launch_ms': t_step * 1e3,
            'peak': fp64_peak, 'peak_source': 'FP64 FMA loop measured live by bench.py (kgeo_measure_fp64_peak)',
            'achieved': None, 'frac': None, 'fp64_flop_per_pixel': POL_FLOP_PER_PIXEL,
            # ncu dram__bytes_read + write of the 160x160 capture scaled by pixels; the capture's
            # outputs (4 MB) stayed in L2, so the writes of a full launch (7 x 3 x 8 B per pixel)
            # are not in it
            'traffic': (1.569e6 + 1.28e3) * npix / 25600,
            'algorithmic_bytes': npix * (16 + norders * 7 * 8 + 2 * 8)}
    if POL_FLOP_PER_PIXEL and fp64_peak:
        roof['achieved'] = POL_FLOP_PER_PIXEL * npix / t_step / 1e12
        roof['frac'] = roof['achieved'] / fp64_peak
        # the FMA loop's peak issues one FP64 instruction per 2 FLOP; dadd / dmul occupy the pipe
        # like a dfma, so the pipe-instruction bound is fp64_peak / 2 instructions per second
        roof['fp64_pipe_frac'] = POL_FP64_INST_PER_PIXEL * npix / t_step / (fp64_peak * 1e12 / 2)
    cpu = None
    if not args.no_cpu_baseline:
        pool, cores = make_pool()  # spawned after the GPU timings
        idx = np.arange(0, npix, max(1, npix // CPU_POL_SAMPLE))[:CPU_POL_SAMPLE]
        chunks = np.array_split(idx, cores * 2)
        t0 = time.time()
        pool.map(_cpu_pol_chunk, [(A[c], B[c]) for c in chunks])
        dt = time.time() - t0
        cpu = {'value': (idx.size / npix) / dt, 'unit': 'images/s', 'cores': cores, 'kind': 'port',
               'sample': '%d pixels (every %dth of the %dx%d image), 3 orders, polarised; oracle/kgeo_oracle.py '
                         'make_image_px on a %d-process pool, %.1f s wall, scaled to the full image'
                         % (idx.size, npix // idx.size, nx, nx, cores, dt)}
        pool.close()
    line = {
        'metric': 'images/s: polarised equatorial image (%dx%d, orders 0..2, I Q U sin(theta_B))' % (nx, nx),
        'value': 1.0 / t_step, 'unit': 'images/s', 'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': t_step * 1e3, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f64', 'data': 'synthetic: make_image pixel grid over [-10, 10] M',
        'config': {'workload': 'reference tests/test_images.py midspin_inclined_subkep: a=0.7, theta_o=45 deg, '
                               'r_o=inf, %dx%d, orders 0..2, ring emissivity, general velocity (xi=0.6, '
                               'beta_phi=0.8, beta_r=0.7), bz_guess field, specind 1' % (nx, nx),
                   'npix': npix, 'orders': norders, 'case': args.case, 'lit_fraction': lit,
                   'l2': 'inputs %d MB, outputs %d MB (compute-bound kernel; not flushed)'
                         % (npix * 16 >> 20, npix * norders * 7 * 8 >> 20)},
        'pixels_per_s': npix / t_step,
        'roofline': roof, 'cpu_baseline': cpu,
        'e2e': {'value': 1.0 / t_e2e, 'unit': 'images/s', 'h2d_bytes_per_step': 2 * 8 * npix,
                'd2h_bytes_per_step': 8 * npix * (7 * norders + 2), 'ms_per_step': t_e2e * 1e3,
                'path': 'kgeo_gb300.equatorial_images.make_image (host grid in, host arrays out)'},
        'gpu_launches': args.steps, 'clocks': ck,
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# curve library: generate_library('rh') of the reference (99 spins x 89 inclinations x
# orders 0..5 x 360 angles, one Brent solve per angle)
# ---------------------------------------------------------------------------

CPU_LIB_SAMPLE = 600     # (curve, angle) roots of the bounded CPU sample
# FP64 work of curve_kernel per root on an ncu capture of the library-small case:
# (dadd + dmul + 2 dfma) thread instructions / roots, and FP64 pipe instructions / roots
LIB_FLOP_PER_ROOT = 153960
LIB_FP64_INST_PER_ROOT = 102000


def roofline_fp64(kernel, t, units, flop_per_unit, inst_per_unit, unit):
    """FP64 roofline object of a compute-bound kernel timed alone: achieved TFLOP/s from the
    captured FLOP per unit, against the FP64 FMA peak measured live; the FP64 pipe's
    instruction rate is fp64_peak / 2 per second."""
    from kgeo_gb300 import device as dev
    peak = dev.fp64_peak_tflops()
    ach = flop_per_unit * units / t / 1e12
    return {'bound': 'fp64', 'unit': 'TFLOP/s', 'kernel': kernel, 'launch_ms': t * 1e3, 'peak': peak,
            'peak_source': 'FP64 FMA loop measured live by bench.py (kgeo_measure_fp64_peak)',
            'achieved': ach, 'frac': ach / peak, 'fp64_flop_per_%s' % unit: flop_per_unit,
            'fp64_pipe_frac': inst_per_unit * units / t / (peak * 1e12 / 2), 'traffic': None,
            'traffic_note': 'compute-bound; inputs and outputs are a few bytes per unit'}


def library_workload(small=False):
    spins = np.linspace(0.01, 0.99, 99)
    incs = np.linspace(1, 89, 89)
    if small:
        spins, incs = spins[::10], incs[::10]
    allincs, allspins = np.meshgrid(incs, spins)
    curves = []
    for sp, inc in zip(allspins.flatten(), allincs.flatten()):
        for m in range(6):
            curves.append((float(sp), float(inc) * np.pi / 180., 1 + np.sqrt(1 - sp * sp), m))
    return curves, np.linspace(-180, 179, 360) * np.pi / 180.


def _cpu_lib_chunk(items):
    from oracle import kgeo_oracle as ko
    from scipy.optimize import brentq
    import warnings
    warnings.filterwarnings('ignore')
    n = 0
    for (a, th0, req, m, vp) in items:
        lo, hi = ko.rho_bracket(m, req)
        try:
            brentq(lambda rho: ko.r_equatorial2(rho, vp, a, th0, mbar=m) - req, lo, hi)
        except (ValueError, RuntimeError):
            pass
        n += 1
    return n


def run_library(args):
    small = args.case == 'library-small'
    pool = cores = None
    import torch
    from kgeo_gb300.equatorial_lensing import rho_of_req_device
    curves, vp = library_workload(small)
    vpd = torch.from_numpy(vp).cuda()
    nroots = len(curves) * vp.size
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    for _ in range(args.warmup):
        rho_of_req_device(curves, vpd)
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    e0, e1 = ev(), ev()
    e0.record(stream)
    for _ in range(args.steps):
        rho, st = rho_of_req_device(curves, vpd)
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    t_step = e0.elapsed_time(e1) / 1e3 / args.steps
    st = st.cpu().numpy()
    # end to end: the public make_library call (angles from the host, tables to the host)
    from kgeo_gb300.equatorial_lensing import make_library
    sp = np.array(sorted({c[0] for c in curves}))
    inc = np.array(sorted({round(c[1] * 180 / np.pi, 9) for c in curves}))
    I, S = np.meshgrid(inc, sp)
    make_library(S.flatten(), I.flatten(), which='rh', mmax=5)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        tabs = make_library(S.flatten(), I.flatten(), which='rh', mmax=5)
    t_e2e = (time.perf_counter() - t0) / args.steps
    cpu = None
    if not args.no_cpu_baseline:
        pool, cores = make_pool()  # spawned after the GPU timings
        rng = np.random.default_rng(0)
        pick = rng.choice(nroots, size=CPU_LIB_SAMPLE, replace=False)
        items = [curves[k // vp.size][:4] + (float(vp[k % vp.size]),) for k in pick]
        chunks = [items[j::cores * 2] for j in range(cores * 2)]
        t0 = time.time()
        pool.map(_cpu_lib_chunk, chunks)
        dt = time.time() - t0
        cpu = {'value': CPU_LIB_SAMPLE / dt, 'unit': 'roots/s', 'cores': cores, 'kind': 'port',
               'sample': '%d random (curve, angle) roots of the same library; oracle/kgeo_oracle.py r_equatorial2 '
                         'under scipy.optimize.brentq (the reference\'s rho_of_req loop) on a %d-process pool, '
                         '%.1f s wall' % (CPU_LIB_SAMPLE, cores, dt)}
        pool.close()
    line = {
        'metric': 'roots/s: curve library (rho_of_req roots, one per curve and angle)',
        'value': nroots / t_step, 'unit': 'roots/s', 'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': t_step * 1e3, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f64', 'data': 'synthetic: the library grid of generate_library',
        'config': {'workload': "generate_library('rh'): %d spins x %d inclinations x orders 0..5 x 360 angles, "
                               'r_eq = r_h, r_o = inf, brentq xtol 2e-12' % (sp.size, inc.size),
                   'curves': len(curves), 'roots': nroots, 'case': args.case,
                   'failed_roots': int((st != 0).sum()), 'l2': 'compute-bound; inputs and outputs < 160 MB'},
        'curves_per_s': len(curves) / t_step,
        'roofline': roofline_fp64('curve_kernel', t_step, nroots, LIB_FLOP_PER_ROOT, LIB_FP64_INST_PER_ROOT,
                                  'root'),
        'cpu_baseline': cpu,
        'e2e': {'value': nroots / t_e2e, 'unit': 'roots/s', 'h2d_bytes_per_step': 8 * vp.size + 48 * len(curves),
                'd2h_bytes_per_step': 12 * nroots, 'ms_per_step': t_e2e * 1e3,
                'path': 'kgeo_gb300.equatorial_lensing.make_library (tables to the host, no files)'},
        'gpu_launches': args.steps, 'clocks': ck,
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# jet field-line crossings (kgeo.solver.findroot) on a traced image
# ---------------------------------------------------------------------------

JET_GRID = 256
JET_CASE = dict(a=0.9, inc=17.0, model='para', psitarget=1.0, ngeo=200, neqmax=1)
CPU_JET_SAMPLE = 2048     # pixels of the bounded CPU sample
# FP64 work of jet_solve_kernel per converged solve on an ncu capture of the jet-small case,
# as for the curve kernel
JET_FLOP_PER_SOLVE = 14310
JET_FP64_INST_PER_SOLVE = 8973


def _cpu_jet_chunk(args):
    A, B = args
    from oracle import kgeo_oracle as ko
    import warnings
    warnings.filterwarnings('ignore')
    c = JET_CASE
    th = c['inc'] * np.pi / 180
    geo = ko.raytrace(c['a'], R_O, th, A, B, c['ngeo'])
    ko.findroot(geo, c['psitarget'], A, B, R_O, th, c['a'], c['ngeo'], model=c['model'], neqmax=c['neqmax'])
    return len(A)


def run_jet(args):
    small = args.case == 'jet-small'
    pool = cores = None
    import torch
    from kgeo_gb300 import device as dev
    from kgeo_gb300 import solver
    from kgeo_gb300.kerr_raytracing_ana import raytrace_ana
    c = JET_CASE
    n = 64 if small else JET_GRID
    x = np.linspace(-10, 10, n)
    A, B = (v.flatten() for v in np.meshgrid(x, x))
    th = c['inc'] * np.pi / 180
    al, be = dev.as_device(A), dev.as_device(B)
    res = dev.trace(c['a'], R_O, th, al, be, ngeo=c['ngeo'])

    class Geo:
        r_s, th_s, mino_times = res['r'], res['th'], res['mino']
    g = solver.getguesses(Geo, c['a'], R_O, th, A, B, c['psitarget'], c['ngeo'], neqmax=c['neqmax'], model=c['model'])
    gd = torch.from_numpy(g).cuda()
    nsolve = int((g != -1).sum())
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    for _ in range(args.warmup):
        solver.findroot_device(c['a'], R_O, th, al, be, gd, c['psitarget'], model=c['model'])
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    e0, e1 = ev(), ev()
    e0.record(stream)
    for _ in range(args.steps):
        out = solver.findroot_device(c['a'], R_O, th, al, be, gd, c['psitarget'], model=c['model'])
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    t_step = e0.elapsed_time(e1) / 1e3 / args.steps
    conv = int(((out['status'] == 0) & (gd != -1)).sum())
    # end to end: numpy pixels in -> raytrace_ana -> findroot -> numpy crossings out
    geo = raytrace_ana(a=c['a'], observer_coords=[0, R_O, th, 0], image_coords=[A, B], ngeo=c['ngeo'], plotdata=False)
    solver.findroot(geo, c['psitarget'], A, B, R_O, th, c['a'], c['ngeo'], model=c['model'], neqmax=c['neqmax'])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        geo = raytrace_ana(a=c['a'], observer_coords=[0, R_O, th, 0], image_coords=[A, B], ngeo=c['ngeo'],
                           plotdata=False)
        solver.findroot(geo, c['psitarget'], A, B, R_O, th, c['a'], c['ngeo'], model=c['model'], neqmax=c['neqmax'])
    t_e2e = (time.perf_counter() - t0) / args.steps
    cpu = None
    if not args.no_cpu_baseline:
        pool, cores = make_pool()  # spawned after the GPU timings
        idx = np.arange(0, A.size, max(1, A.size // CPU_JET_SAMPLE))[:CPU_JET_SAMPLE]
        chunks = np.array_split(idx, cores * 2)
        t0 = time.time()
        pool.map(_cpu_jet_chunk, [(A[k], B[k]) for k in chunks])
        dt = time.time() - t0
        cpu = {'value': idx.size / dt, 'unit': 'pixels/s (trace + findroot)', 'cores': cores, 'kind': 'port',
               'sample': '%d pixels (every %dth of the %dx%d grid): oracle raytrace + findroot (scipy newton) on a '
                         '%d-process pool, %.1f s wall' % (idx.size, A.size // idx.size, n, n, cores, dt)}
        pool.close()
    line = {
        'metric': 'crossing solves/s: jet field-line crossings (findroot secant per guess)',
        'value': nsolve / t_step, 'unit': 'solves/s', 'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': t_step * 1e3, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f64', 'data': 'synthetic: uniform image-plane grid over [-10, 10] M',
        'config': {'workload': 'a=0.9, theta_o=17 deg, r_o=1e4, %dx%d, ngeo=200, BZ paraboloid psi=1, neqmax=1' % (n, n),
                   'guesses': list(g.shape), 'solves': nsolve, 'converged': conv, 'case': args.case,
                   'l2': 'compute-bound (per-ray records 624 B / pixel)'},
        'roofline': roofline_fp64('jet_solve_kernel', t_step, nsolve, JET_FLOP_PER_SOLVE, JET_FP64_INST_PER_SOLVE,
                                  'solve'),
        'cpu_baseline': cpu,
        'e2e': {'value': A.size / t_e2e, 'unit': 'pixels/s (trace + findroot)', 'h2d_bytes_per_step': 16 * A.size,
                'd2h_bytes_per_step': 48 * c['ngeo'] * A.size + 48 * g.size, 'ms_per_step': t_e2e * 1e3,
                'path': 'raytrace_ana + kgeo_gb300.solver.findroot (numpy in/out)'},
        'gpu_launches': args.steps, 'clocks': ck,
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# jet Stokes images (kgeo.off_eq.getstokes, the BZ monopole field line)
# ---------------------------------------------------------------------------

STOKES_GRID = 256
STOKES_CASE = dict(a=0.5, inc=60.0, model='mono', psitarget=0.4, ngeo=200, neqmax=1, nu_parallel=0.0, sigma=2.0)
CPU_STOKES_SAMPLE = 2048
# FP64 work of jet_stokes_kernel per crossing (r != 0) on an ncu capture of the stokes-small
# case: dadd + dmul + 2 dfma, and FP64 pipe instructions
STOKES_FLOP_PER_CROSSING = 2940
STOKES_FP64_INST_PER_CROSSING = 1901


def _cpu_stokes_chunk(args):
    A, B = args
    from oracle import kgeo_oracle as ko
    import warnings
    warnings.filterwarnings('ignore')
    c = STOKES_CASE
    with np.errstate(all='ignore'):
        ko.getstokes_mono(c['psitarget'], A, B, R_O, c['inc'] * np.pi / 180, c['a'], c['ngeo'], neqmax=c['neqmax'],
                          model=c['model'], nu_parallel=c['nu_parallel'], sigma=c['sigma'], table=True)
    return len(A)


def run_stokes(args):
    small = args.case == 'stokes-small'
    pool = cores = None
    import torch
    from kgeo_gb300 import device as dev
    from kgeo_gb300 import off_eq, solver
    c = STOKES_CASE
    n = 64 if small else STOKES_GRID
    x = np.linspace(-10, 10, n)
    A2, B2 = np.meshgrid(x, x)
    A, B = A2.flatten(), B2.flatten()
    th = c['inc'] * np.pi / 180
    al, be = dev.as_device(A), dev.as_device(B)
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def pipeline():
        geo = dev.trace(c['a'], R_O, th, al, be, ngeo=c['ngeo'], outputs=('r', 'th', 'mino'), per_ray=())
        cr, shape = solver.crossings_device(c['a'], R_O, th, al, be, geo['r'], geo['th'], geo['mino'],
                                            c['psitarget'], model=c['model'], neqmax=c['neqmax'])
        return cr, off_eq.stokes_device(c['a'], R_O, th, al, be, cr, neqmax=c['neqmax'], model=c['model'],
                                        nu_parallel=c['nu_parallel'], sigma=c['sigma'])
    for _ in range(args.warmup):
        cr, st = pipeline()
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    e0, e1 = ev(), ev()
    e0.record(stream)
    for _ in range(args.steps):
        cr, st = pipeline()
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    t_step = e0.elapsed_time(e1) / 1e3 / args.steps
    G = cr['r'].shape[0]
    # the emission kernel alone, on the step's crossings
    e2, e3 = ev(), ev()
    e2.record(stream)
    for _ in range(args.steps):
        off_eq.stokes_device(c['a'], R_O, th, al, be, cr, neqmax=c['neqmax'], model=c['model'],
                             nu_parallel=c['nu_parallel'], sigma=c['sigma'])
    e3.record(stream)
    torch.cuda.synchronize()
    t_kern = e2.elapsed_time(e3) / 1e3 / args.steps
    ncross = int((cr['r'] != 0).sum())
    # end to end: numpy pixels in -> getstokes -> numpy images out
    kw = dict(model=c['model'], neqmax=c['neqmax'], nu_parallel=c['nu_parallel'], sigma=c['sigma'])
    off_eq.getstokes(c['psitarget'], A2, B2, R_O, th, c['a'], c['ngeo'], **kw)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        off_eq.getstokes(c['psitarget'], A2, B2, R_O, th, c['a'], c['ngeo'], **kw)
    t_e2e = (time.perf_counter() - t0) / args.steps
    cpu = None
    if not args.no_cpu_baseline:
        pool, cores = make_pool()  # spawned after the GPU timings
        idx = np.arange(0, A.size, max(1, A.size // CPU_STOKES_SAMPLE))[:CPU_STOKES_SAMPLE]
        chunks = np.array_split(idx, cores * 2)
        # the density's stagnation radius comes from the first crossing of the first guess row:
        # every chunk starts with the image's first crossing pixel so that it has one
        i0 = int(torch.nonzero(cr['r'][0] != 0)[0, 0])
        t0 = time.time()
        pool.map(_cpu_stokes_chunk, [(np.r_[A[i0], A[k]], np.r_[B[i0], B[k]]) for k in chunks])
        dt = time.time() - t0
        cpu = {'value': idx.size / dt, 'unit': 'pixels/s (getstokes)', 'cores': cores, 'kind': 'port',
               'sample': '%d pixels (every %dth of the %dx%d grid) in %d chunks, each led by the image\'s first '
                         'crossing pixel: oracle getstokes (raytrace, findroot, emission) on a %d-process pool, '
                         '%.1f s wall' % (idx.size, A.size // idx.size, n, n, len(chunks), cores, dt)}
        pool.close()
    roof = roofline_fp64('jet_stokes_kernel', t_kern, ncross, STOKES_FLOP_PER_CROSSING, STOKES_FP64_INST_PER_CROSSING,
                         'crossing')
    roof['timed'] = 'kgeo_jet_stokes: jet_stagnation_kernel (one block) + jet_stokes_kernel'
    line = {
        'metric': 'pixels/s: jet Stokes images (getstokes: trace, field-line crossings, emission, subring sums)',
        'value': A.size / t_step, 'unit': 'pixels/s', 'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': t_step * 1e3, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f64', 'data': 'synthetic: uniform image-plane grid over [-10, 10] M',
        'config': {'workload': 'a=0.5, theta_o=60 deg, r_o=1e4, %dx%d, ngeo=200, BZ monopole psi=0.4, neqmax=1, '
                               'nu_parallel=0, sigma=2' % (n, n),
                   'guess_rows': G, 'crossings': ncross, 'case': args.case,
                   'stokes_kernel_ms': t_kern * 1e3, 'l2': 'per-step buffers 24 B x ngeo x pixels'},
        'roofline': roof,
        'cpu_baseline': cpu,
        'e2e': {'value': A.size / t_e2e, 'unit': 'pixels/s (getstokes)', 'h2d_bytes_per_step': 16 * A.size,
                'd2h_bytes_per_step': 32 * (c['neqmax'] + 1) * A.size, 'ms_per_step': t_e2e * 1e3,
                'path': 'kgeo_gb300.off_eq.getstokes (numpy in/out)'},
        'gpu_launches': args.steps * 12, 'clocks': ck,
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# configuration 4: batched images (64 images, one persistent launch, CUDA graph)
# ---------------------------------------------------------------------------

BATCH_IMAGES = 64


def batch_workload(n_img=BATCH_IMAGES, small=False):
    """64 images from default_rng(0): side ~ U{128..768} (uniform integer), a ~ U[0, 0.998),
    theta_o ~ U[1, 89] deg, ngeo ~ U{64, 128, 256}, grids over [-12, 12] M."""
    rng = np.random.default_rng(0)
    ims, A, B = [], [], []
    for _ in range(n_img):
        side = int(rng.integers(128, 769))
        if small:
            side = max(8, side // 8)
        a = float(rng.uniform(0, 0.998))
        th = float(rng.uniform(1, 89)) * np.pi / 180
        ng = int(rng.choice([64, 128, 256]))
        x = np.linspace(-12, 12, side)
        Ai, Bi = np.meshgrid(x, x)
        ims.append(dict(a=a, th_o=th, npix=side * side, ngeo=ng, side=side))
        A.append(Ai.flatten())
        B.append(Bi.flatten())
    return ims, np.concatenate(A), np.concatenate(B)


def _oracle_batch_chunk(args):
    a, th_o, A, B, G = args
    from oracle import kgeo_oracle as ko
    import warnings
    warnings.filterwarnings('ignore')
    ko.raytrace(a, R_O, th_o, A, B, G)
    return len(A)


def run_batch(args, emit=True):
    small = args.case == 'batch-small'
    pool = cores = None
    import torch
    from kgeo_gb300 import device as dev
    from kgeo_gb300.batch import BatchPlan
    ims, A, B = batch_workload(small=small)
    n_rays = A.size
    keys = ('t', 'r', 'th', 'ph', 'sig')
    plan = BatchPlan(ims, precision='mixed', keys=keys)
    al, be = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    plan.bind(al, be)
    t0 = time.perf_counter()
    cfg = plan.autotune(budget_ms=3000)
    t_tune = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    for _ in range(args.warmup):
        plan.graph_launch()
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    e0, e1 = ev(), ev()
    e0.record(stream)
    for _ in range(args.steps):
        plan.graph_launch()
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    t_mixed = e0.elapsed_time(e1) / 1e3 / args.steps
    n_points = plan.n_samples
    # FP64 recurrence on the same batch (same plan shape, own outputs after the mixed ones
    # are checked) and the plain FP64 kernel (independent evaluation per sample) on every 8th
    # image, scaled by points
    sub = list(range(0, len(ims), 8))
    off = np.cumsum([0] + [im['npix'] for im in ims])
    errs = {k: {'max': 0.0, 'rms_sum': 0.0, 'n': 0} for k in keys}
    t_plain, pts_plain = 0.0, 0
    for i in sub:
        im = ims[i]
        sl = slice(int(off[i]), int(off[i + 1]))
        prep = dev.PreparedRays(im['a'], R_O, im['th_o'], al[sl], be[sl], ngeo=im['ngeo'])
        out = prep.alloc(keys=keys)
        prep.samples(out, chunk=cfg['chunk'])
        got = plan.image(i)
        for k in keys:
            # the scales of the configuration-3 statistics: relative, with a floor of 1 rad for
            # the angles and of r_o for t and sigma
            x, y = got[k], out[k]
            floor = {'r': 1e-300, 'th': 1.0, 'ph': 1.0, 't': R_O, 'sig': R_O}[k]
            d = (x - y).abs() / y.abs().clamp_min(floor)
            d = d[torch.isfinite(d)]
            if d.numel():
                errs[k]['max'] = max(errs[k]['max'], float(d.max()))
                errs[k]['rms_sum'] += float((d * d).sum())
                errs[k]['n'] += int(d.numel())
        torch.cuda.synchronize()
        a0, a1 = ev(), ev()
        a0.record(stream)
        # the same pipeline as the batch's: per-ray setup, then the samples
        prep.setup()
        prep.samples(out, chunk=0)
        a1.record(stream)
        torch.cuda.synchronize()
        t_plain += a0.elapsed_time(a1) / 1e3
        pts_plain += im['npix'] * im['ngeo']
        del out, prep
    mixed_err = {k: {'max': v['max'], 'rms': float(np.sqrt(v['rms_sum'] / max(v['n'], 1)))} for k, v in errs.items()}
    plain_pts_per_s = pts_plain / t_plain
    pts_per_ray = n_points / n_rays
    plan_d = BatchPlan(ims, precision='fp64', keys=('r',))
    plan_d.bind(al, be)
    plan_d.run()
    torch.cuda.synchronize()
    e0.record(stream)
    plan_d.run()
    e1.record(stream)
    torch.cuda.synchronize()
    t_fp64 = e0.elapsed_time(e1) / 1e3
    plan_d.close()
    cpu = None
    if not args.no_cpu_baseline:
        pool, cores = make_pool()  # spawned after the GPU timings
        rng = np.random.default_rng(0)
        idx = np.sort(rng.choice(n_rays, n_rays // 256, replace=False))
        img_of = np.searchsorted(off, idx, side='right') - 1
        jobs = []
        for i in np.unique(img_of):
            sel = idx[img_of == i]
            for c in np.array_split(sel, max(1, sel.size // 512)):
                jobs.append((ims[i]['a'], ims[i]['th_o'], A[c], B[c], ims[i]['ngeo']))
        tc0 = time.time()
        pool.map(_oracle_batch_chunk, jobs)
        dt = time.time() - tc0
        pool.close()
        cpu = {'value': idx.size / dt, 'unit': 'rays/s', 'cores': cores, 'kind': 'port',
               'sample': '%d rays (seeded 1/256 of the batch, every image proportionally, its own ngeo); '
                         'oracle/kgeo_oracle.py raytrace on a %d-process pool, %.1f s wall' % (idx.size, cores, dt)}
    line = {
        'metric': 'Kerr rays/s: 64 batched images, mixed precision, one persistent launch in a CUDA graph',
        'value': n_rays / t_mixed, 'unit': 'rays/s', 'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': t_mixed * 1e3, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f32+f64', 'data': 'synthetic: 64 image-plane grids from default_rng(0)',
        'config': {'workload': 'configuration 4: 64 images, side ~ U{128..768}, a ~ U[0, 0.998), theta_o ~ '
                               'U[1, 89] deg, ngeo ~ U{64, 128, 256}, grids over [-12, 12] M, r_o = 1e4',
                   'rays': n_rays, 'samples': n_points, 'precision': 'mixed', 'case': args.case,
                   'tuned': cfg, 'tune_s': t_tune, 'l2': 'outputs %.0f GB per step' % (n_points * 40 / 1e9)},
        'points_per_s': n_points / t_mixed,
        'fp64_batched_recurrence': {'value': n_rays / t_fp64, 'ms_per_step': t_fp64 * 1e3},
        'fp64_plain': {'value': plain_pts_per_s / pts_per_ray, 'points_per_s': plain_pts_per_s,
                       'sample': 'images %s, per-ray setup + independent evaluation per sample (the batch '
                                 'pipeline\'s stages), scaled by points' % sub},
        'speedup_vs_fp64_plain': (n_rays / t_mixed) / (plain_pts_per_s / pts_per_ray),
        'speedup_vs_fp64_recurrence': t_fp64 / t_mixed,
        'mixed_vs_fp64_error': mixed_err,
        'cpu_baseline': cpu, 'clocks': ck, 'gpu_launches': 6 * args.steps,
    }
    plan.close()
    if emit:
        print(json.dumps(line))
    return line


def main():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=5)
    p.add_argument('--warmup', type=int, default=3)
    p.add_argument('--impl', choices=('ours', 'reference'), default='ours')
    p.add_argument('--case', choices=('full', 'small', 'mixed', 'mixed-small', 'image', 'image-small', 'batch',
                                      'batch-small', 'polimage', 'polimage-small', 'library', 'library-small', 'jet',
                                      'jet-small', 'stokes', 'stokes-small'),
                   default='full')
    p.add_argument('--no-cpu-baseline', action='store_true')
    p.add_argument('--no-extras', action='store_true', help='skip the other configurations (the configurations key)')
    args = p.parse_args()
    if args.impl == 'reference':
        run_reference(args)
    elif args.case.startswith('mixed'):
        run_mixed(args)
    elif args.case.startswith('image'):
        run_image(args)
    elif args.case.startswith('polimage'):
        run_polimage(args)
    elif args.case.startswith('library'):
        run_library(args)
    elif args.case.startswith('jet'):
        run_jet(args)
    elif args.case.startswith('stokes'):
        run_stokes(args)
    elif args.case.startswith('batch'):
        run_batch(args)
    else:
        run_ours(args)


if __name__ == '__main__':
    main()
