"""Benchmark of the elastic velocity-stress hot path on GB300.

Workload: one time step (stress sweep, stress ghosts, velocity sweep,
velocity ghosts, source) of the 9-field elastic staggered-grid scheme on a
512^3 interior grid, space order 4, FP32, seeded layered heterogeneous medium
(20 layers, vp U[1.5,4.5] km/s, 5% smoothed perturbation, vs = vp/sqrt(3),
Gardner density), 10 m spacing, 15 Hz Ricker source, dt = 0.5 x stable step.
All inputs are synthetic and seeded.  The 18 field levels + 8 media arrays
(~15 GB) are far larger than L2, so no explicit flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

``--scheme acoustic`` measures the regular-grid (acoustic) scheme instead: the
reference's tests/simplewaveequation.py model (one field, three time levels,
its initialisation) on a 512^3 interior, space order 4, FP32; one step is one
sweep (12 B of algorithmic traffic per grid point).

Prints one JSON line.  Under torchrun each rank runs an independent replica
(the path has no exchange step); value is the sum over ranks of grid-point
updates divided by the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, 'opesci-fd_gb300')):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = 'elastic GLUP/s (grid-point updates of all 9 fields per second), 512^3 SO4 FP32 heterogeneous'
UNIT = 'GLUP/s'
# algorithmic bytes per grid point of each sweep (FP32 fields, FP32 media):
# stress reads U V W + 6 stresses + lambda mu mu12 mu13 mu23, writes 6 stresses
# (80 B); velocity reads U V W + 6 stresses + beta (beta1..3 are formed from
# beta and its neighbours on the fly), writes U V W (52 B).  The reference's
# formulation, with beta1..3 as three arrays, needs 140 B per point.
STRESS_BYTES_PER_LUP = 4 * (9 + 5 + 6)
VELOCITY_BYTES_PER_LUP = 4 * (9 + 1 + 3)
STEP_BYTES_PER_LUP = STRESS_BYTES_PER_LUP + VELOCITY_BYTES_PER_LUP


def dist_env():
    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', '1'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return rank, world, local


def measured_peak():
    p = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d['hbm_gbs']), 'measured (MEASURED_PEAKS.json hbm_gbs)'
    return 6800.0, 'fallback 6.8 TB/s'


def profiled_traffic(kind):
    """DRAM bytes per grid point of a kernel from the committed ncu summary
    (profiles/traffic.txt lines '<kernel> <bytes_per_lup>'), or None."""
    p = os.path.join(ROOT, 'profiles', 'traffic.txt')
    if not os.path.exists(p):
        return None
    for line in open(p):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kind:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


class ClockSampler(object):
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed
    region (200 ms period)."""

    FIELDS = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix='.csv')
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.FIELDS,
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(',')]
            if len(p) >= 8:
                rows.append(p)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[0]) for r in rows if r[0].replace('.', '').isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[i] for r in rows for i in range(4) if r[4 + i].lower() == 'active'})
        return {'sm_mhz': statistics.median(sm) if sm else None,
                'sm_max_mhz': max(mx) if mx else None,
                'reasons': reasons, 'samples': len(rows)}


def build_problem(n, so, steps, seed=0):
    from opesci.models import layered_problem
    return layered_problem(n, space_order=so, ntsteps=steps, seed=seed)


def cpu_flags(vectorize):
    return '-O3 -fopenmp' if vectorize else '-g -O3 -fno-tree-vectorize -fopenmp'


def cpu_model():
    """Host CPU model name (lscpu, else /proc/cpuinfo), for the baseline record."""
    try:
        out = subprocess.run(['lscpu'], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith('model name'):
                return line.split(':', 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open('/proc/cpuinfo'):
            if line.lower().startswith('model name'):
                return line.split(':', 1)[1].strip()
    except OSError:
        pass
    return 'unknown'


def elastic_config(n, so, storage, world, variant, footprint_gb=None):
    """The config dict both arms print for the elastic workload."""
    return {'workload': 'elastic %d^3 SO%d %s heterogeneous + Ricker source, free surfaces'
                        % (n, so, storage.upper()),
            'grid': [n, n, n], 'space_order': so, 'storage': storage,
            'parallelism': 'replicas x%d' % world,
            'l2_flush': 'inputs larger than L2' + (' (%.1f GB resident)' % footprint_gb if footprint_gb else ''),
            'kernel_variant': variant}


def cpu_baseline_pair(n, so, steps, threads=None):
    """Both CPU builds of the oracle program on the same bounded sample: the
    stated baseline is g++ -O3 -fopenmp (vectorisation on); the reference's
    own GNU flags (-fno-tree-vectorize) are reported beside it."""
    v_vec, cores, s_vec = cpu_oracle(n, so, steps, threads=threads, vectorize=True)
    v_ref, _, s_ref = cpu_oracle(n, so, steps, threads=threads, vectorize=False)
    return {'value': v_vec, 'unit': UNIT, 'cores': cores, 'kind': 'port',
            'cpu_model': cpu_model(), 'omp_proc_bind': 'close',
            'sample': '%d steps of a %d^3 problem of the same kind (SO%d, heterogeneous, source), '
                      'reference-shaped generated C++ (g++ -O3 -fopenmp), time loop only, %.1f s'
                      % (steps, n, so, s_vec),
            'reference_flags': {'value': v_ref, 'flags': cpu_flags(False), 'seconds': s_ref}}


def cpu_oracle(n, so, steps, seed=0, threads=None, vectorize=False):
    """Time the reference-shaped generated C++ (the oracle program: the
    reference's generator output for this model, reference GNU flags) on the
    host cores for ``steps`` steps of an n^3 problem of the same kind."""
    from opesci.models import layered_problem
    from oracle import run as orun
    with tempfile.TemporaryDirectory() as d:
        files = {k: os.path.join(d, k + '.raw') for k in ('rho', 'vp', 'vs')}
        g, media, src, wav = layered_problem(n, space_order=so, ntsteps=steps, seed=seed, media_files=files)
        out = orun.run(g, d, source=(src, wav), threads=threads, dump=False, vectorize=vectorize)
    lups = float(n) ** 3 * steps
    return lups / out['loop_seconds'] / 1e9, out['threads'], out['loop_seconds']


def link_bandwidth(nbytes):
    """Plain pinned-host <-> device copy bandwidth (GB/s) of one buffer of
    ``nbytes``: the host link this box gives a single cudaMemcpyAsync, the
    ceiling of the end-to-end transfers."""
    import torch
    h = torch.empty(nbytes // 4, dtype=torch.float32, pin_memory=True)
    h.zero_()
    d = torch.empty_like(h, device='cuda')
    out = {}
    for name, (dst, src) in (('h2d', (d, h)), ('d2h', (h, d))):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(3):
            dst.copy_(src, non_blocking=True)
        e1.record()
        torch.cuda.synchronize()
        out[name] = 3 * nbytes / (e0.elapsed_time(e1) / 1e3) / 1e9
    del d, h
    return out


def pinned(shape, keep):
    """A float32 array in page-locked host memory.  The torch tensor that
    owns the memory goes into ``keep``, which the caller holds while the
    array is in use: the array's memory does not keep the tensor alive, and
    once the tensor is gone torch's host allocator takes the block back
    (copies into such an array measured 20-35 GB/s against 180 GB/s)."""
    import torch
    t = torch.empty(shape, dtype=torch.float32, pin_memory=True)
    keep.append(t)
    return t.numpy()


def elastic_e2e(sim, media, src, wav, steps, lups):
    """One job through the C ABI as a user runs it: media from pinned host
    memory in (with the effective-media preprocessing), ``steps`` steps, the
    nine final fields out to pinned host memory, all in the timed region (one
    wait at the end).  After one warm-up job, the median of three jobs is
    the value; a phase-timed job after them gives the transfer rates,
    against the plain copy bandwidth of the host link."""
    import numpy as np
    keep = []   # owners of the pinned buffers, alive until the jobs are done
    pin = lambda: pinned(sim.dims, keep)  # noqa: E731
    host_media = []
    for arr in media:
        hb = pin()
        hb[...] = arr
        host_media.append(hb)
    host_fields = [pin() for _ in range(9)]
    for hb in host_fields:   # first touch of the pinned output pages outside the timed region
        hb[...] = 0.0
    cells = float(np.prod(sim.dims))

    def job(k, phases=None):
        sim.sync()
        t0 = time.perf_counter()
        sim.zero()
        sim.steps = 0
        sim.set_media_async(*host_media)
        if phases is not None:
            sim.sync()
            phases['media_s'] = time.perf_counter() - t0
        sim.set_source(src, wav)
        sim.step(k)
        if phases is not None:
            sim.sync()
            phases['steps_s'] = time.perf_counter() - t0 - phases['media_s']
        t1 = time.perf_counter()
        sim.download_all_async(host_fields, level=k % 2)
        sim.sync()
        t2 = time.perf_counter()
        if phases is not None:
            phases['download_s'] = t2 - t1
        return t2 - t0

    job(steps)   # warm-up: first DMA use of the pinned buffers, the library's scratch pool
    walls = sorted(job(steps) for _ in range(3))
    wall = walls[1]
    phases = {}
    job(steps, phases)
    link = link_bandwidth(int(cells) * 4)
    return {'value': lups / wall / 1e9, 'unit': UNIT,
            'jobs_s': walls,
            'h2d_bytes_per_step': (3 * cells * 4 + len(wav) * 4) / steps,
            'd2h_bytes_per_step': 9 * cells * 4 / steps,
            'seconds': wall,
            'phases_s': phases,
            'media_upload_GBps': 3 * cells * 4 / phases['media_s'] / 1e9,
            'field_download_GBps': 9 * cells * 4 / phases['download_s'] / 1e9,
            'link_GBps': link,
            'note': 'one job through the C ABI from pinned host buffers: media upload + effective media, '
                    'K steps, download of the 9 final fields (one wait at the end); median of 3 jobs after '
                    'a warm-up job; media_upload_GBps includes the effective-media preprocessing; '
                    'link_GBps is a plain pinned copy'}


def run_reference(args, rank):
    """The reference arm: the oracle program (the reference-shaped generated
    C++) on the bench's own workload, all host threads, both builds: g++ -O3
    -fopenmp (the stated value) and the reference's GNU flags beside it."""
    if rank != 0:
        return
    n = args.size if args.ref_size is None else args.ref_size
    steps = max(1, min(args.steps, args.ref_steps))
    vec = not args.cpu_reference_flags
    val, cores, secs = cpu_oracle(n, args.space_order, steps, vectorize=vec)
    other = None
    if not args.cpu_single_build:
        v2, _, s2 = cpu_oracle(n, args.space_order, steps, vectorize=not vec)
        other = {'value': v2, 'flags': cpu_flags(not vec), 'seconds': s2}
    base = {'value': val, 'unit': UNIT, 'cores': cores, 'kind': 'port', 'cpu_model': cpu_model(),
            'omp_proc_bind': 'close',
            'sample': '%d steps of the %d^3 problem, reference-shaped generated C++ (g++ %s), time loop only'
                      % (steps, n, cpu_flags(vec))}
    if other:
        base['reference_flags' if vec else 'vectorized'] = other
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': val, 'unit': UNIT,
        'n_gpus': args.gpus, 'steps': steps, 'warmup': 0, 'ms_per_step': secs * 1e3 / steps,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': args.storage,
        'data': 'synthetic (seeded layered medium, Ricker source)',
        'config': elastic_config(args.size, args.space_order, args.storage, args.gpus, args.variant),
        'cpu_baseline': base,
        'e2e': {'value': val, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line), flush=True)


ACOUSTIC_METRIC = 'acoustic GLUP/s (grid-point updates per second), 512^3 SO4 FP32 regular grid'
# reads u[t] and u[t-1], writes u[t+1]
ACOUSTIC_BYTES_PER_LUP = 3 * 4


def acoustic_problem(n, so, steps):
    """The reference's acoustic model on an n^3 interior (unit cube split in
    n intervals, grid_size n-1), its two initial levels: level 0 = 0 and
    level 1 = v*dt on the interior (the reference's initialisation with
    v = 1 on a zero level 0)."""
    import numpy as np
    from opesci.models import simplewave_grid
    h = 1.0 / (n - 1)
    g = simplewave_grid(grid_size=(n - 1,) * 3, dt=0.4 * h / (3 ** 0.5 * 2), tmax=1.0, space_order=so,
                        ntsteps=steps)
    dims = tuple(d.value for d in g.dim)
    m = g.margin.value
    l1 = np.zeros(dims, dtype=np.float32)
    l1[m:-m, m:-m, m:-m] = np.float32(np.float32(1.0) * np.float32(g.dt.value))
    return g, l1


def acoustic_cpu(n, so, steps, threads=None, vectorize=False):
    from oracle import run as orun
    from opesci.models import simplewave_grid
    with tempfile.TemporaryDirectory() as d:
        g = simplewave_grid(grid_size=(n - 1,) * 3, dt=0.4 / (n - 1) / (3 ** 0.5 * 2), tmax=1.0,
                            space_order=so, ntsteps=steps)
        out = orun.run_regular(g, d, threads=threads, dump=False, vectorize=vectorize)
    return float(n) ** 3 * steps / out['loop_seconds'] / 1e9, out['threads'], out['loop_seconds']


def run_acoustic(args, rank, world, local):
    import numpy as np
    from opesci import runtime, replicas

    n, so = args.size, args.space_order
    if args.impl == 'reference':
        if rank != 0:
            return
        steps = max(1, min(args.steps, args.ref_steps))
        val, cores, secs = acoustic_cpu(n, so, steps, vectorize=args.cpu_vectorize)
        line = {'impl': 'reference', 'metric': ACOUSTIC_METRIC, 'value': val, 'unit': UNIT,
                'n_gpus': args.gpus, 'steps': steps, 'warmup': 0, 'ms_per_step': secs * 1e3 / steps,
                'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
                'data': 'synthetic (the reference acoustic model and initialisation)',
                'config': {'workload': 'acoustic %d^3 SO%d FP32' % (n, so), 'grid': [n, n, n], 'space_order': so},
                'cpu_baseline': {'value': val, 'unit': UNIT, 'cores': cores, 'kind': 'port',
                                 'sample': '%d steps, reference-shaped generated C++ (g++ %s), time loop only'
                                           % (steps, cpu_flags(args.cpu_vectorize))},
                'e2e': {'value': val, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
        print(json.dumps(line), flush=True)
        return

    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group('nccl')
    runtime.set_device(local)
    g, l1 = acoustic_problem(n, so, args.warmup + args.steps)
    sim = runtime.RegularSimulation(runtime.regular_config_from_grid(g, variant=args.variant))
    sim.upload(1, l1)
    sim.step(args.warmup)
    sim.sync()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if dist is not None:
        dist.barrier()
    sim.sync()
    total_ms = sim.step_timed(args.steps)
    if dist is not None:
        dist.barrier()
    clocks = sampler.stop()
    lups_rank = float(n) ** 3 * args.steps
    rate, secs = replicas.aggregate_rate(lups_rank, total_ms / 1e3, dist, device='cuda')
    ms = secs * 1e3
    peak, peak_src = measured_peak()
    launch_ms = total_ms / args.steps
    bytes_launch = float(n) ** 3 * ACOUSTIC_BYTES_PER_LUP
    achieved = bytes_launch / (launch_ms / 1e3) / 1e9
    tr = profiled_traffic('regular_sweep_so%d_f32_v%d' % (so, args.variant))
    roofline = {'bound': 'hbm', 'kernel': 'regular sweep (%s)' % ('direct', 'shared-memory ring')[args.variant],
                'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                'frac': achieved / peak, 'peak_source': peak_src,
                'traffic': (tr * float(n) ** 3) if tr else None,
                'algorithmic_bytes_per_launch': bytes_launch, 'avg_launch_ms': launch_ms}
    e2e = None
    if not args.no_e2e:
        keep = []   # owners of the pinned buffers, alive until the jobs are done
        h0, h1, hout = (pinned(sim.dims, keep) for _ in range(3))
        h0[...] = 0.0
        h1[...] = l1
        hout[...] = 0.0

        def job():
            sim.sync()
            t0 = time.perf_counter()
            sim.steps = 0
            sim.upload(0, h0)
            sim.upload(1, h1)
            sim.step(args.steps)
            sim.lib.ofd_regular_download(sim.h, sim.newest_level(), hout.ctypes.data)
            sim.sync()
            return time.perf_counter() - t0

        job()   # warm-up: first DMA use of the pinned buffers
        walls = sorted(job() for _ in range(3))
        wall = walls[1]
        cells = float(np.prod(sim.dims))
        e2e = {'value': lups_rank / wall / 1e9, 'unit': UNIT, 'jobs_s': walls,
               'h2d_bytes_per_step': 2 * cells * 4 / args.steps, 'd2h_bytes_per_step': cells * 4 / args.steps,
               'note': 'through the C ABI from pinned host buffers: two initial levels in, K steps, '
                       'the newest level out; median of 3 jobs after a warm-up job'}
    sim.close()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            # the bench's own grid, fewer steps (about 10 s on 16 cores)
            csteps = max(1, min(args.cpu_steps, 100))
            v, cores, csecs = acoustic_cpu(n, so, csteps)
            cpu = {'value': v, 'unit': UNIT, 'cores': cores, 'kind': 'port',
                   'sample': '%d steps of the %d^3 acoustic model, reference-shaped generated C++ '
                             '(g++ -g -O3 -fno-tree-vectorize -fopenmp), time loop only, %.1f s'
                             % (csteps, n, csecs)}
        except Exception as e:  # report, do not hide
            cpu = {'value': None, 'error': str(e)[:300]}
    if rank == 0:
        line = {'metric': ACOUSTIC_METRIC, 'value': rate / 1e9, 'unit': UNIT, 'n_gpus': world,
                'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': ms / args.steps,
                'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
                'data': 'synthetic (the reference acoustic model and initialisation)',
                'config': {'workload': 'acoustic %d^3 SO%d FP32 regular grid' % (n, so), 'grid': [n, n, n],
                           'space_order': so, 'parallelism': 'replicas x%d' % world,
                           'l2_flush': 'inputs larger than L2 (3 levels, %.1f GB)'
                                       % (3 * float(np.prod(sim.dims)) * 4 / 1e9),
                           'kernel_variant': args.variant},
                'roofline': roofline, 'cpu_baseline': cpu, 'e2e': e2e, 'clocks': clocks,
                'gpu_launches': args.steps}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=200)
    ap.add_argument('--warmup', type=int, default=5)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--size', type=int, default=512)
    ap.add_argument('--space-order', type=int, default=4)
    ap.add_argument('--storage', default='f32')
    ap.add_argument('--variant', type=int, default=0)
    ap.add_argument('--ref-size', type=int, default=None)
    ap.add_argument('--ref-steps', type=int, default=10)
    ap.add_argument('--cpu-size', type=int, default=256)
    ap.add_argument('--cpu-steps', type=int, default=200)   # ~10 s of CPU work at 256^3
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--scheme', default='elastic', choices=['elastic', 'acoustic'])
    # reference arm: the stated value is the g++ -O3 -fopenmp build (the
    # reference's generated C++ as "g++ -O3, OpenMP"); --cpu-reference-flags
    # states the reference's own -fno-tree-vectorize build instead, and
    # --cpu-single-build skips timing the other build beside it
    ap.add_argument('--cpu-reference-flags', action='store_true')
    ap.add_argument('--cpu-single-build', action='store_true')
    ap.add_argument('--cpu-vectorize', action='store_true', help=argparse.SUPPRESS)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()

    if args.scheme == 'acoustic':
        run_acoustic(args, rank, world, local)
        return

    if args.impl == 'reference':
        run_reference(args, rank)
        return

    import numpy as np
    from opesci import runtime

    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group('nccl')
    runtime.set_device(local)   # libofd carries its own CUDA runtime

    n, so = args.size, args.space_order
    g, media, src, wav = build_problem(n, so, args.warmup + args.steps)
    cfg = runtime.config_from_grid(g, storage=args.storage, kernel_variant=args.variant)
    sim = runtime.Simulation(cfg)
    sim.set_coefficients_from_grid(g)
    sim.set_media(*media)
    sim.set_source(src, wav)
    sim.step(args.warmup)
    sim.sync()

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if dist is not None:
        dist.barrier()
    sim.sync()
    # timed region: K steps on the launch path, CUDA events on the handle's
    # stream around each kernel class of every step (the roofline's kernel
    # times) and from the first to the last (the value)
    total_ms, cls_ms, launches = sim.step_profiled(args.steps)
    sim.sync()
    if dist is not None:
        dist.barrier()
    clocks = sampler.stop()
    prof_steps = args.steps
    from opesci import replicas
    lups_rank = float(n) ** 3 * args.steps
    rate, secs = replicas.aggregate_rate(lups_rank, total_ms / 1e3, dist, device='cuda')
    ms = secs * 1e3
    value = rate / 1e9

    peak, peak_src = measured_peak()
    stress_ms = cls_ms[0] / prof_steps
    vel_ms = cls_ms[2] / prof_steps
    esz = {'f32': 4, 'f16': 2, 'bf16': 2, 'f64': 8}.get(args.storage, 4)
    sb = (9 + 6) * esz + 5 * 4
    vb = (9 + 3) * esz + 4
    stress_bytes = float(n) ** 3 * sb
    achieved = stress_bytes / (stress_ms / 1e3) / 1e9
    tr = profiled_traffic('stress_sweep_so%d_%s' % (so, args.storage))
    roofline = {'bound': 'hbm', 'kernel': 'stress sweep', 'achieved': achieved, 'peak': peak,
                'unit': 'GB/s', 'frac': achieved / peak, 'peak_source': peak_src,
                'traffic': (tr * float(n) ** 3) if tr else None,
                'algorithmic_bytes_per_launch': stress_bytes,
                'avg_launch_ms': stress_ms,
                'velocity_sweep': {'achieved': float(n) ** 3 * vb / (vel_ms / 1e3) / 1e9, 'avg_launch_ms': vel_ms},
                'step': {'bytes_per_lup': sb + vb,
                         'achieved': float(n) ** 3 * (sb + vb) * args.steps / (ms / 1e3) / 1e9},
                'class_ms_per_step': [c / prof_steps for c in cls_ms],
                'classes_from': 'the timed region: CUDA events around each kernel class of each of its %d steps'
                                % prof_steps}

    if so == 4:
        # the stress sweep alone: at space order 4 the generated ghosts'
        # FP64 recompute runs beside it in the step (its FP64 work shares
        # the SM with the sweep); a short profiled pass with the recompute
        # moved after the sweep shows the kernel by itself
        k = min(args.steps, 20)
        sim.set_ghost_schedule(0, 8)
        _, cls2, _ = sim.step_profiled(k)
        sim.set_ghost_schedule(1, 4)   # back to the library's default schedule
        alone = cls2[0] / k
        roofline['stress_sweep_alone'] = {
            'avg_launch_ms': alone, 'achieved': stress_bytes / (alone / 1e3) / 1e9,
            'frac': stress_bytes / (alone / 1e3) / 1e9 / peak,
            'recompute_after_sweep_ms': cls2[1] / k,
            'note': 'profiled pass of %d steps after the timed region with the ghost recompute after the '
                    'sweep (ofd_set_ghost_schedule(0, 8)); class 1 then holds the recompute' % k}

    e2e = None
    if not args.no_e2e:
        e2e = elastic_e2e(sim, media, src, wav, args.steps, lups_rank)
    sim.close()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline_pair(args.cpu_size, so, args.cpu_steps)
        except Exception as e:  # report, do not hide
            cpu = {'value': None, 'error': str(e)[:300]}

    if rank == 0:
        line = {
            'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': ms / args.steps, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': args.storage,
            'data': 'synthetic (seeded layered medium, Ricker source)',
            'config': elastic_config(n, so, args.storage, world, args.variant),
            'l2_flush_detail': 'inputs larger than L2: %.1f GB resident' % (runtime.Simulation.footprint(cfg) / 1e9),
            'roofline': roofline, 'cpu_baseline': cpu, 'e2e': e2e, 'clocks': clocks,
            'gpu_launches': launches,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
