"""Benchmark: steps/s and ms per Newton iteration of the IPC Newton loop on the 960k-tet twisted bar.

Workload: a 0.05 x 0.05 x 1.0 m bar, 20 x 20 x 400 hexes x 6 tets (176,841 vertices, 960,000
tets), Neo-Hookean E = 1e6 Pa, nu = 0.45, rho = 1000, d-hat = 5e-4 m, dt = 0.01 s, both end faces
Dirichlet and rotating at +-pi rad/s, seed-drawn +-1e-4 m jitter: synthetic data generated here.
A step is one implicit time step (the full Newton loop with CCD line search).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--nx 400]

Ours: W warm-up steps, then K steps timed with CUDA events on the simulation stream between a
barrier + synchronize on both sides (max over ranks); `value` = N*K / max time.  Nothing inside
the timed region records per-launch events.  `e2e` re-runs the same K steps from the same state
through the C-ABI path with the state copied from pinned host memory before each step and read
back after it.  The roofline comes from a separate instrumented pass over the same steps (CUDA
events around every launch of the profiled kernel).  `trajectory` times the whole 200-step run of
the scene from t = 0 and the CPU oracle on single steps taken from its states at steps 50, 100
and 150.  With --gpus N > 1 (torchrun) every rank runs an independent replica: the path has no
data-parallel shard (one scene, one GPU).

Reference arm (--impl reference): the CPU oracle's implementation of the same Newton path
(C/OpenMP kernels + block-Jacobi PCG, all host cores), timed on whole time steps of the same
scene; rank 0 only.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = 'steps/s (twisted bar, 960k tets)'


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--nx', type=int, default=400, help='hexes along the bar (400 = the 960k-tet configuration)')
    ap.add_argument('--pcg-rtol', type=float, default=1e-6)
    ap.add_argument('--warm-start', type=int, default=1, help='PCG initial guess from the previous step (1) or zero (0)')
    ap.add_argument('--profile-kernel', type=int, default=1, help='kernel timed for the roofline (1 = PCG SpMV)')
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--precond', default='multigrid', choices=['multigrid', 'two-level'],
                    help='PCG preconditioner of the bar, lattice and cube workloads')
    ap.add_argument('--mg-smoothing', default='fp32', choices=['fp64', 'fp32'],
                    help="precision of the multigrid V-cycle's two level-0 smoothing products")
    ap.add_argument('--cpu-sample-pcg', type=int, default=100000)
    ap.add_argument('--workload', default='bar', choices=['bar', 'batch', 'lattice', 'cubes', 'stack2d', 'admm', 'direct'],
                    help='bar: the 960k-tet twisted bar (headline); batch: 512 independent cube stacks in one context; '
                         'lattice: 216 cubes dropped on a ground box; cubes: two 8^3-hex cubes; '
                         'stack2d: the 2D path, 16 squares of 16x16 quads on a ground segment; '
                         'admm: the ADMM-IPC variant on the two-cube drop; '
                         'direct: the direct (multifrontal Cholesky) solve of the lattice\'s Newton system at first contact')
    ap.add_argument('--scenes', type=int, default=512, help='scenes of the batch workload')
    ap.add_argument('--learned-steps', type=int, default=20,
                    help='steps run from the timed state with the inertial and the learned start (0: skip)')
    ap.add_argument('--learned-weights', default=os.path.join(HERE, 'fastipc_gb300', 'weights', 'warmstart_bar400.npz'))
    ap.add_argument('--trajectory', type=int, default=200,
                    help='bar: time the whole run of this many steps from t = 0 beside the K-step window (0: skip)')
    ap.add_argument('--cpu-samples', default='50,100,150',
                    help='trajectory steps whose GPU states the CPU oracle steps once each (empty: none)')
    return ap.parse_args()


def make_scene(args):
    from fastipc_gb300 import scenes
    if args.workload == 'lattice':
        return scenes.cube_lattice(m=6, n=6, seed=0)
    if args.workload == 'cubes':
        return scenes.two_cubes(n=8, seed=0)
    nx = args.nx
    return scenes.twisted_bar(nx=nx, ny=20, nz=20, size=(nx / 400.0, 0.05, 0.05), seed=0)


def metric(args):
    return {'lattice': 'steps/s (216-cube lattice drop, 280k tets)', 'cubes': 'steps/s (two cubes, 6k tets)'}.get(args.workload, METRIC)


def workload(args):
    common = {'newton_tol': '|p|inf < 1e-2 dt', 'pcg_rtol': args.pcg_rtol, 'pcg_tolerance': 'relative to |rhs| on free DOFs'}
    if args.workload == 'lattice':
        return dict(common, workload='6x6x6 lattice of 0.1 m cubes (6 hexes per side x6 tets), seed-drawn rotations and +-10% '
                                     'jitter, dropped on a fixed 2x0.1x2 m ground box; NH E=1e5 nu=0.4, dhat=1e-3, dt=0.01',
                    tets=279942, verts=74096, l2='inputs larger than L2 (element Hessians alone ~0.2 GB per Newton iteration)')
    if args.workload == 'cubes':
        return dict(common, workload='two 0.1 m cubes of 8x8x8 hexes x6 tets, upper one rotated (seed 0) and moving at -1 m/s; '
                                     'NH E=1e5 nu=0.4, dhat=1e-3, dt=0.01', tets=6144, verts=1458,
                    l2='working set smaller than L2, not flushed between steps (a 6k-tet scene is bound by launches and '
                       'host syncs, not by memory)')
    nx = args.nx
    return dict(common, workload=f'twisted bar {nx}x20x20 hexes x6 tets ({nx * 2400} tets), NH E=1e6 nu=0.45, dhat=5e-4, dt=0.01',
                tets=nx * 2400, verts=(nx + 1) * 441, l2='inputs larger than L2 (element Hessians alone ~0.7 GB per Newton iteration)')


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix='.csv')
        os.close(fd)
        q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,'
             'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')
        try:
            self.proc = subprocess.Popen(['nvidia-smi', f'--id={self.index}', f'--query-gpu={q}', '--format=csv,noheader,nounits',
                                          '-lms', '200'], stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        import statistics
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(',')]
                if len(f) >= 9 and f[1].isdigit():
                    rows.append(f)
        except OSError:
            pass
        if not rows:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unsampled']}
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == 'active'})
        return {'sm_mhz': statistics.median(int(r[1]) for r in rows), 'sm_max_mhz': int(rows[0][2]),
                'power_w_max': max(float(r[3]) for r in rows if r[3].replace('.', '').isdigit()) if rows else None,
                'reasons': reasons, 'samples': len(rows)}


def peaks():
    try:
        return json.load(open(os.path.join(HERE, 'MEASURED_PEAKS.json'))), 'measured'
    except (OSError, ValueError):
        return {'hbm_gbs': 6800.0, 'bf16_tflops': 1900.0}, 'fallback'


def ncu_traffic(kernel_id):
    """dram bytes per launch of the profiled kernel from a committed ncu capture, if any."""
    name = {1: 'pcg_spmv', 2: 'pcg_update', 3: 'nh_element'}.get(kernel_id)
    path = os.path.join(HERE, 'profiles', f'{name}_traffic.json')
    try:
        d = json.load(open(path))
        return float(d['dram_bytes_per_launch_scaled']), d.get('note')
    except (OSError, ValueError, KeyError):
        return None, None


def fp64_peak(dev):
    """Measured FP64 FMA throughput of this GPU (TFLOP/s): the library's probe kernel (8
    independent FMA chains per thread, 8 CTAs of 256 threads per SM), best of 5 launches timed
    with CUDA events on the launching stream."""
    import torch
    from fastipc_gb300 import _native
    L = _native.lib()
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks, iters = 8 * nsm, 8192
    out = torch.empty(blocks * 256, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = _native.stream()

    def launch():
        _native.check(L.fipc_fp64_fma_probe(blocks, iters, _native.dptr(out), sp), 'fipc_fp64_fma_probe')
    launch()
    best = float('inf')
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        launch()
        e1.record(stream)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    flops = blocks * 256 * iters * 16.0
    return {'tflops': flops / (best / 1e3) / 1e12, 'ms': best, 'flops': flops,
            'how': f'k_fp64_fma_probe: {blocks} CTAs x 256 threads x {iters} rounds x 8 FMA chains, best of 5 (CUDA events)'}


def snapshot(sim):
    return (sim.x.clone(), sim.v.clone(), sim.dx_prev.clone(), {k: v.clone() for k, v in sim._dir_hist.items()})


def restore(sim, snap):
    sim.x.copy_(snap[0])
    sim.v.copy_(snap[1])
    sim.dx_prev.copy_(snap[2])
    sim._dir_hist = {k: v.clone() for k, v in snap[3].items()}


def cpu_baseline(scene, newton_per_step, pcg_per_newton, args, spmv_per_iter=1):
    """The oracle on the host cores: one Newton iteration of time step 1 of the same scene
    (constraints, assembly, full PCG solve, line search), scaled to steps/s with the Newton
    iteration count of the timed GPU steps.  `value`: the CPU credited with the GPU's PCG
    iteration count times the fine-level products each GPU iteration makes (spmv_per_iter: 1 for
    block-Jacobi or the two-level preconditioner, 3 for a multigrid V(1,1)-cycle), at the cost of
    its own block-Jacobi iterations; `own_solver_value`: its own block-Jacobi PCG to the same
    tolerance."""
    from oracle import oracle as O
    sim = O.OracleSim(scene, solver='bsr', pcg_rtol=args.pcg_rtol, pcg_maxit=args.cpu_sample_pcg)
    sim.step(0, max_newton=1)                 # rest state (zero right-hand side)
    sim.timings = {}
    t0 = time.perf_counter()
    sim.compute_xn_and_xTilde()
    sim.move_nodes(1 * sim.dt)
    sim.find_constraints()
    sim.compute_hessian_and_gradient()
    t1 = time.perf_counter()
    sim.solve_system(1 * sim.dt)
    t2 = time.perf_counter()
    E0 = sim.compute_energy()
    sim.xPrev = sim.x.copy()
    alpha = sim.compute_intersection_free_step_size()
    sim.apply_sol(alpha)
    sim.check_collision()
    sim.find_constraints()
    sim.compute_energy()
    t3 = time.perf_counter()
    pcg_its = max(sim.pcg_iters[-1], 1)
    t_fixed = (t1 - t0) + (t3 - t2)
    t_pcg_it = (t2 - t1) / pcg_its
    t_newton = t_fixed + t_pcg_it * pcg_per_newton * spmv_per_iter
    sps = 1.0 / (t_newton * newton_per_step)
    t_own = t_fixed + t_pcg_it * pcg_its
    _ = E0
    return {'value': sps, 'unit': 'steps/s', 'cores': O.lib().oracle_num_threads(), 'kind': 'port',
            'sample': (f'one Newton iteration of step 1 of the same scene on the host cores ({t3 - t0:.1f} s: '
                       f'assembly+constraints+line search {t_fixed:.2f} s, PCG {pcg_its} its at {1e3 * t_pcg_it:.2f} ms/it); '
                       f'scaled by the timed GPU steps\' {newton_per_step:.2f} Newton its/step and {pcg_per_newton:.0f} PCG its/Newton '
                       f'x {spmv_per_iter} fine-level products each'),
            'ms_per_newton_iter': 1e3 * t_newton,
            'matched_iterations': ('value: the CPU is credited with the GPU\'s PCG iteration count times the fine-level '
                                   'matrix products of each GPU iteration, at the cost of one of its own block-Jacobi '
                                   'iterations per product'),
            'own_solver_value': 1.0 / (t_own * newton_per_step),
            'own_solver': (f'the oracle\'s own block-Jacobi PCG ({pcg_its} its per Newton iteration in the sample), the '
                           f'solver the reference arm (--impl reference) runs'),
            'own_solver_ms_per_newton_iter': 1e3 * t_own}


def max_over_ranks(ms, dist, device):
    """The slowest rank's time (ms) of a timed region: an all-reduce MAX over the ranks (the
    value itself for one process)."""
    if dist is None:
        return float(ms)
    import torch
    t = torch.tensor([float(ms)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, steps, ms_max):
    """Whole-job steps/s of `world` independent replicas that each ran `steps` steps, timed by
    the slowest one."""
    return world * steps / (ms_max / 1e3)


def run_reference(args):
    """CPU oracle, whole time steps of the same scene (rank 0 only)."""
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    from oracle import oracle as O
    scene = make_scene(args)
    sim = O.OracleSim(scene, solver='bsr', pcg_rtol=args.pcg_rtol, pcg_maxit=args.cpu_sample_pcg)
    f = 0
    for _ in range(args.warmup):
        sim.step(f)
        f += 1
    t0 = time.perf_counter()
    n0 = len(sim.newton_iters)
    for _ in range(args.steps):
        sim.step(f)
        f += 1
    dt = time.perf_counter() - t0
    its = sim.newton_iters[n0:]
    v = args.steps / dt
    out = {'impl': 'reference', 'metric': metric(args), 'value': v, 'unit': 'steps/s', 'n_gpus': args.gpus, 'steps': args.steps,
           'warmup': args.warmup, 'ms_per_step': 1e3 * dt / args.steps, 'higher_is_better': True, 'scaling': 'weak',
           'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'config': workload(args),
           'ms_per_newton_iter': 1e3 * dt / max(sum(its), 1), 'newton_iters_per_step': sum(its) / len(its),
           'cpu_baseline': {'value': v, 'unit': 'steps/s', 'cores': O.lib().oracle_num_threads(), 'kind': 'port',
                            'sample': f'{args.steps} whole time steps ({args.warmup}..{args.warmup + args.steps - 1}) of the same scene'},
           'e2e': {'value': v, 'unit': 'steps/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.workload == 'batch':
        return main_batch(args)
    if args.workload == 'stack2d':
        return main_2d(args)
    if args.workload == 'direct':
        return main_direct(args)
    if args.workload == 'admm':
        return main_admm(args)
    if args.impl == 'reference':
        return run_reference(args)
    import numpy as np
    import torch
    from fastipc_gb300 import _native
    from fastipc_gb300.build import build
    from fastipc_gb300.newton import NewtonIPC

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl')
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    build()
    scene = make_scene(args)
    sim = NewtonIPC(scene, device=dev, pcg_rtol=args.pcg_rtol, pcg_warm_start=bool(args.warm_start))
    if args.precond == 'two-level':
        sim.set_preconditioner(2048)
    sim.set_multigrid_fp32(args.mg_smoothing == 'fp32')
    mg = sim.multigrid()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)

    f = 0
    for _ in range(args.warmup):
        sim.step(f)
        f += 1
    snap = snapshot(sim)
    f0 = f
    n_newton0, n_pcg0 = len(sim.newton_iters), len(sim.pcg_iters)
    L = _native.lib()
    L.fipc_profile_enable(0)                  # no per-launch events inside the timed region
    stream = torch.cuda.current_stream(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = _native.launch_count()
    barrier()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            sim.step(f)
            f += 1
        ev1.record(stream)
        barrier()
    launches = _native.launch_count() - launches0
    ms = ev0.elapsed_time(ev1)
    newton = sim.newton_iters[n_newton0:]
    pcg = sim.pcg_iters[n_pcg0:]
    ms_max = max_over_ranks(ms, dist, dev)
    value = replica_throughput(world, args.steps, ms_max)

    # e2e: the same steps again from the same state, state round-tripped through pinned host memory
    hx = torch.empty_like(snap[0], device='cpu').pin_memory()
    hv = torch.empty_like(snap[1], device='cpu').pin_memory()
    hx.copy_(snap[0])
    hv.copy_(snap[1])
    restore(sim, snap)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    f = f0
    for _ in range(args.steps):
        sim.x.copy_(hx, non_blocking=True)
        sim.v.copy_(hv, non_blocking=True)
        sim.step(f)
        hx.copy_(sim.x, non_blocking=True)
        hv.copy_(sim.v, non_blocking=True)
        f += 1
    e1.record(stream)
    barrier()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1), dist, dev)
    nbytes = 2 * sim.x.numel() * 8

    # roofline: a separate instrumented pass over the first steps of the same window, with a CUDA
    # event pair around every launch of the profiled kernel
    restore(sim, snap)
    n_prof = min(args.steps, 5)
    barrier()
    L.fipc_profile_enable(args.profile_kernel)
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for k in range(n_prof):
        sim.step(f0 + k)
    p1.record(stream)
    barrier()
    pt, pn, pb, pf = ctypes_read(L)
    L.fipc_profile_enable(0)
    prof_ms = p0.elapsed_time(p1)

    learned = learned_leg(sim, snap, f0, args) if args.learned_steps > 0 and args.workload == 'bar' else None
    traj = trajectory_leg(sim, scene, args, dev) if args.trajectory > 0 and args.workload == 'bar' else None

    if rank == 0:
        pk, src = peaks()
        fp64 = fp64_peak(dev)
        achieved = pb / (pt / 1e3) / 1e9 if pt > 0 else None
        achieved_tf = pf / (pt / 1e3) / 1e12 if pt > 0 else None
        traffic, note = ncu_traffic(args.profile_kernel)
        newton_per_step = sum(newton) / len(newton)
        pcg_per_newton = sum(pcg) / max(len(pcg), 1)
        hbm = {'achieved': achieved, 'peak': pk['hbm_gbs'], 'unit': 'GB/s', 'frac': achieved / pk['hbm_gbs'] if achieved else None,
               'peak_source': f'{src} (MEASURED_PEAKS.json hbm_gbs)' if src == 'measured' else 'fallback 6.8 TB/s'}
        f64 = {'achieved': achieved_tf, 'peak': fp64['tflops'], 'unit': 'TFLOP/s',
               'frac': achieved_tf / fp64['tflops'] if achieved_tf else None, 'peak_source': 'measured: ' + fp64['how']}
        kname = {1: 'k_pcg_spmv', 2: 'k_pcg_update', 3: 'k_elasticity'}.get(args.profile_kernel)
        # the binding unit of the profiled kernel, from its ncu capture: the FP64 pipe (SpMV 80%
        # busy against 39% DRAM; update 62% against 21%; Neo-Hookean element 90% against 5%)
        roof = {'kernel': kname, 'bound': 'fp64', 'achieved': achieved_tf, 'peak': fp64['tflops'], 'unit': 'TFLOP/s',
                'frac': f64['frac'], 'traffic': traffic * 1.0 if traffic is not None else None,
                'algorithmic_bytes_per_launch': pb / max(pn, 1), 'algorithmic_flops_per_launch': pf / max(pn, 1),
                'avg_launch_us': 1e3 * pt / max(pn, 1), 'launches': pn, 'hbm': hbm, 'fp64': f64,
                'binding': 'fp64 pipe (ncu: profiles/pcg_spmv_twisted_bar_960k.md)',
                'measured_in': f'instrumented pass over steps {f0}..{f0 + n_prof - 1} after the timed region',
                'time_share_of_step': pt / prof_ms if prof_ms > 0 else None}
        if note:
            roof['traffic_note'] = note
        cfg = workload(args)
        cfg['preconditioner'] = (f'multigrid V(1,1), {mg["levels"]} levels of {mg["nodes"]} nodes, '
                                 f'{args.mg_smoothing.upper()} level-0 smoothing products' if mg['levels']
                                 else 'two-level additive (rigid-body modes of 2048-vertex runs)')
        out = {'metric': metric(args), 'value': value, 'unit': 'steps/s', 'n_gpus': world, 'steps': args.steps,
               'warmup': args.warmup, 'ms_per_step': ms_max / args.steps, 'higher_is_better': True, 'scaling': 'weak',
               'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'config': cfg,
               'ms_per_newton_iter': ms_max / max(sum(newton), 1), 'newton_iters_per_step': newton_per_step,
               'pcg_iters_per_newton': pcg_per_newton, 'parallelism': 'replicas' if world > 1 else 'single',
               'e2e': {'value': world * args.steps / (e2e_ms / 1e3), 'unit': 'steps/s', 'h2d_bytes_per_step': nbytes,
                       'd2h_bytes_per_step': nbytes},
               'gpu_launches': launches, 'roofline': roof, 'clocks': clk.summary(),
               'sections_s': {k: round(v, 4) for k, v in sim.timer.total.items()}}
        if traj:
            out['trajectory'] = traj
        if learned:
            out['learned_warm_start'] = learned
        if world == 1 and not args.no_cpu_baseline:
            out['cpu_baseline'] = cpu_baseline(scene, newton_per_step, pcg_per_newton, args, 3 if mg['levels'] else 1)
            if traj and traj.get('gpu_states') is not None:
                traj.update(trajectory_cpu(scene, traj.pop('gpu_states'), args))
        if traj:
            traj.pop('gpu_states', None)
        print(json.dumps(out), flush=True)
    sim.close()
    if dist is not None:
        dist.destroy_process_group()


def trajectory_leg(sim, scene, args, dev):
    """The scene's whole run of args.trajectory steps from t = 0 (the initial state, an empty
    PCG warm-start history), device-timed with one CUDA event per step; keeps the GPU states at
    the --cpu-samples steps (device copies) for the CPU comparison."""
    import torch
    n = args.trajectory
    samples = sorted({int(t) for t in args.cpu_samples.split(',') if t.strip() and 0 <= int(t) < n})
    sim.set_state(scene.initial_positions(), scene.v)
    sim.dx_prev.zero_()
    sim._dir_hist = {}
    stream = torch.cuda.current_stream(dev)
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(n + 1)]
    states, newton, pcg = {}, [], []
    torch.cuda.synchronize(dev)
    evs[0].record(stream)
    for f in range(n):
        if f in samples:
            states[f] = (sim.x.clone(), sim.v.clone())
        p0 = len(sim.pcg_iters)
        newton.append(sim.step(f))
        pcg.append(sum(sim.pcg_iters[p0:]))
        evs[f + 1].record(stream)
    torch.cuda.synchronize(dev)
    step_ms = [evs[f].elapsed_time(evs[f + 1]) for f in range(n)]
    total = sum(step_ms)
    out = {'steps': n, 'value': n / (total / 1e3), 'unit': 'steps/s', 'ms_per_step': total / n,
           'newton_iters_per_step': sum(newton) / n, 'ms_per_newton_iter': total / max(sum(newton), 1),
           'pcg_iters_per_newton': sum(pcg) / max(sum(newton), 1), 'how': 'device-timed (CUDA events), whole run from t = 0',
           'per_quarter': []}
    q = max(n // 4, 1)
    for a in range(0, n, q):
        b = min(a + q, n)
        out['per_quarter'].append({'steps': f'{a}..{b - 1}', 'steps_per_s': (b - a) / (sum(step_ms[a:b]) / 1e3),
                                   'newton_iters_per_step': sum(newton[a:b]) / (b - a)})
    out['gpu_states'] = {f: (x.cpu().numpy(), v.cpu().numpy(), step_ms[f], newton[f], pcg[f]) for f, (x, v) in states.items()}
    return out


def trajectory_cpu(scene, states, args):
    """The CPU oracle (all host cores, its own block-Jacobi PCG) takes one step from each of the
    GPU's states, the same step the GPU took there; per-step rates on those steps, as measured
    (own solver) and with the CPU credited with the GPU's PCG iteration count."""
    from oracle import oracle as O
    if not states:
        return {}
    sim = O.OracleSim(scene, solver='bsr', pcg_rtol=args.pcg_rtol, pcg_maxit=args.cpu_sample_pcg)
    rows, g_ms, c_ms, c_ms_m = [], 0.0, 0.0, 0.0
    for f in sorted(states):
        x, v, gms, gnewton, gpcg = states[f]
        sim.x, sim.v = x.copy(), v.copy()
        sim.timings = {}
        p0 = len(sim.pcg_iters)
        t0 = time.perf_counter()
        it = sim.step(f)
        dt = time.perf_counter() - t0
        cpcg = sum(sim.pcg_iters[p0:])
        t_solve = sim.timings.get('Solve System', 0.0)
        matched = dt - t_solve + (t_solve / max(cpcg, 1)) * gpcg
        rows.append({'step': f, 'gpu_ms': gms, 'gpu_newton': gnewton, 'gpu_pcg': gpcg, 'cpu_ms': 1e3 * dt, 'cpu_newton': it,
                     'cpu_pcg': cpcg, 'cpu_ms_matched_iterations': 1e3 * matched})
        g_ms += gms
        c_ms += 1e3 * dt
        c_ms_m += 1e3 * matched
    n = len(rows)
    return {'cpu_samples': rows, 'cpu_cores': O.lib().oracle_num_threads(),
            'gpu_steps_per_s_on_samples': n / (g_ms / 1e3), 'cpu_steps_per_s_on_samples': n / (c_ms / 1e3),
            'cpu_steps_per_s_on_samples_matched_iterations': n / (c_ms_m / 1e3)}


BATCH_METRIC = 'scene-steps/s (cube stacks, batched)'


def batch_workload(n):
    return {'workload': f'{n} independent cube stacks (1-8 cubes of 3-10 hexes per side x6 tets over a fixed ground box, '
                        f'seeds 0..{n - 1}), NH E=1e5 nu=0.4, dhat=1e-3, dt=0.01, one batch context',
            'scenes': n, 'newton_tol': '|p|inf < 1e-2 dt per scene', 'l2': 'inputs larger than L2'}


def main_batch(args):
    """Batched scenes: W warm-up steps, K timed steps of all scenes (CUDA events), value =
    scenes * K / time; the oracle steps a sample of the same scenes on the host cores."""
    rank = int(os.environ.get('RANK', '0'))
    from fastipc_gb300 import scenes as SC
    scs = SC.cube_stacks(args.scenes, seed=0)
    n_tets = sum(s.n_tets for s in scs)
    cfg = batch_workload(args.scenes)
    cfg.update({'tets': n_tets, 'verts': sum(s.n_verts for s in scs), 'pcg_rtol': args.pcg_rtol})
    if args.impl == 'reference':
        if rank != 0:
            return
        v, sample, cores = batch_cpu(scs, args)
        print(json.dumps({'impl': 'reference', 'metric': BATCH_METRIC, 'value': v, 'unit': 'scene-steps/s', 'n_gpus': args.gpus,
                          'steps': args.steps, 'warmup': args.warmup, 'higher_is_better': True, 'scaling': 'weak',
                          'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'config': cfg,
                          'cpu_baseline': {'value': v, 'unit': 'scene-steps/s', 'cores': cores, 'kind': 'port', 'sample': sample},
                          'e2e': {'value': v, 'unit': 'scene-steps/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}),
              flush=True)
        return
    import torch
    from fastipc_gb300 import _native
    from fastipc_gb300.batch import BatchNewtonIPC
    from fastipc_gb300.build import build
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    build()
    t0 = time.perf_counter()
    sim = BatchNewtonIPC(scs, device=dev, pcg_rtol=args.pcg_rtol)
    t_setup = time.perf_counter() - t0
    f = 0
    for _ in range(args.warmup):
        sim.step(f)
        f += 1
    snap = (sim.x.clone(), sim.v.clone())
    f0 = f
    n0 = len(sim.newton_iters)
    stream = torch.cuda.current_stream(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = _native.launch_count()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            sim.step(f)
            f += 1
        ev1.record(stream)
        torch.cuda.synchronize(dev)
    launches = _native.launch_count() - launches0
    ms = ev0.elapsed_time(ev1)
    its = sim.newton_iters[n0:]
    newton_rounds = sum(int(i.max()) for i in its)
    # e2e: the same steps from the same state with the state round-tripped through pinned host memory
    hx = torch.empty_like(snap[0], device='cpu').pin_memory()
    hv = torch.empty_like(snap[1], device='cpu').pin_memory()
    hx.copy_(snap[0])
    hv.copy_(snap[1])
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    f = f0
    for _ in range(args.steps):
        sim.x.copy_(hx, non_blocking=True)
        sim.v.copy_(hv, non_blocking=True)
        sim.step(f)
        hx.copy_(sim.x, non_blocking=True)
        hv.copy_(sim.v, non_blocking=True)
        f += 1
    e1.record(stream)
    torch.cuda.synchronize(dev)
    e2e_ms = e0.elapsed_time(e1)
    nbytes = 2 * sim.x.numel() * 8
    out = {'metric': BATCH_METRIC, 'value': args.scenes * args.steps / (ms / 1e3), 'unit': 'scene-steps/s', 'n_gpus': 1,
           'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': ms / args.steps, 'higher_is_better': True, 'scaling': 'weak',
           'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'config': cfg,
           'newton_iters_per_scene_step': float(sum(i.mean() for i in its) / len(its)),
           'batched_newton_rounds_per_step': newton_rounds / len(its), 'ms_per_batched_newton_round': ms / max(newton_rounds, 1),
           'pcg_shape': sim.pcg_shape(), 'setup_s': t_setup,
           'e2e': {'value': args.scenes * args.steps / (e2e_ms / 1e3), 'unit': 'scene-steps/s', 'h2d_bytes_per_step': nbytes,
                   'd2h_bytes_per_step': nbytes},
           'gpu_launches': launches, 'clocks': clk.summary(), 'sections_s': {k: round(v, 4) for k, v in sim.timer.total.items()}}
    if not args.no_cpu_baseline:
        v, sample, cores = batch_cpu(scs, args)
        out['cpu_baseline'] = {'value': v, 'unit': 'scene-steps/s', 'cores': cores, 'kind': 'port', 'sample': sample}
    print(json.dumps(out), flush=True)
    sim.close()


STACK2D_METRIC = 'steps/s (2D: 16 squares, 8k triangles)'


def main_2d(args):
    """The 2D path (NEWTON_IPC.py with dim == 2): a column of 16 squares of 16 x 16 quads x2
    triangles (4,626 vertices, 8,192 triangles, the size of the reference's 2D testcases) dropped
    on a fixed ground segment; W warm-up
    steps, K timed steps (CUDA events), e2e with the state through pinned host memory; the 2D
    oracle times whole steps of the same scene from the same state on the host."""
    from fastipc_gb300 import scenes as SC
    rank = int(os.environ.get('RANK', '0'))
    scene = SC.square_stack_2d(k=16, n=16, seed=0)
    cfg = {'workload': '2D: 16 squares of 16x16 quads x2 fixed-corotated triangles on a ground segment (4626 verts, '
                       '8192 tris), E=1e5 nu=0.4, dhat=1e-3, dt=0.01', 'tris': int(len(scene.tris)), 'verts': int(len(scene.x)),
           'pcg_rtol': args.pcg_rtol, 'newton_tol': '|p|inf < 1e-2 dt',
           'l2': 'working set smaller than L2, not flushed between steps (the 2D step is bound by launch and barrier latency)'}

    def cpu_steps(x0, v0, f0, budget_s=20.0):
        from oracle import oracle2d as O2
        o = O2.OracleSim2D(scene, fast=True)
        o.x, o.v = x0.copy(), v0.copy()
        t0 = time.perf_counter()
        n = 0
        while n < args.steps and (n == 0 or time.perf_counter() - t0 < budget_s):
            o.step(f0 + n)
            n += 1
        dt = time.perf_counter() - t0
        return n / dt, (f'{n} whole time steps ({f0}..{f0 + n - 1}) of the same scene from the same state (C + OpenMP '
                        f'element, constraint, CCD and intersection loops; scipy assembly and sparse LU)')

    if args.impl == 'reference':
        if rank != 0:
            return
        from oracle import oracle2d as O2
        o = O2.OracleSim2D(scene, fast=True)
        for f in range(args.warmup):
            o.step(f)
        v, sample = cpu_steps(o.x, o.v, args.warmup)
        print(json.dumps({'impl': 'reference', 'metric': STACK2D_METRIC, 'value': v, 'unit': 'steps/s', 'n_gpus': args.gpus,
                          'steps': args.steps, 'warmup': args.warmup, 'higher_is_better': True, 'scaling': 'weak',
                          'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'config': cfg,
                          'cpu_baseline': {'value': v, 'unit': 'steps/s', 'cores': O2.O.lib().oracle_num_threads(), 'kind': 'port',
                                           'sample': sample},
                          'e2e': {'value': v, 'unit': 'steps/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}), flush=True)
        return
    import torch
    from fastipc_gb300 import _native
    from fastipc_gb300.build import build
    from fastipc_gb300.newton2d import NewtonIPC2D
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    build()
    sim = NewtonIPC2D(scene, device=dev, pcg_rtol=args.pcg_rtol)
    f = 0
    for _ in range(args.warmup):
        sim.step(f)
        f += 1
    snap = (sim.x.clone(), sim.v.clone())
    f0, n0 = f, len(sim.newton_iters)
    stream = torch.cuda.current_stream(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = _native.launch_count()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            sim.step(f)
            f += 1
        ev1.record(stream)
        torch.cuda.synchronize(dev)
    launches = _native.launch_count() - launches0
    ms = ev0.elapsed_time(ev1)
    its = sim.newton_iters[n0:]
    hx = torch.empty_like(snap[0], device='cpu').pin_memory()
    hv = torch.empty_like(snap[1], device='cpu').pin_memory()
    hx.copy_(snap[0])
    hv.copy_(snap[1])
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    f = f0
    for _ in range(args.steps):
        sim.x.copy_(hx, non_blocking=True)
        sim.v.copy_(hv, non_blocking=True)
        sim.step(f)
        hx.copy_(sim.x, non_blocking=True)
        hv.copy_(sim.v, non_blocking=True)
        f += 1
    e1.record(stream)
    torch.cuda.synchronize(dev)
    e2e_ms = e0.elapsed_time(e1)
    nbytes = 2 * sim.x.numel() * 8
    out = {'metric': STACK2D_METRIC, 'value': args.steps / (ms / 1e3), 'unit': 'steps/s', 'n_gpus': 1, 'steps': args.steps,
           'warmup': args.warmup, 'ms_per_step': ms / args.steps, 'higher_is_better': True, 'scaling': 'weak',
           'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'config': cfg,
           'newton_iters_per_step': sum(its) / len(its), 'ms_per_newton_iter': ms / max(sum(its), 1),
           'pcg_iters_per_newton': sum(sim.pcg_iters[-sum(its):]) / max(sum(its), 1),
           'e2e': {'value': args.steps / (e2e_ms / 1e3), 'unit': 'steps/s', 'h2d_bytes_per_step': nbytes, 'd2h_bytes_per_step': nbytes},
           'gpu_launches': launches, 'clocks': clk.summary(), 'sections_s': {k: round(v, 4) for k, v in sim.timer.total.items()}}
    if not args.no_cpu_baseline:
        v, sample = cpu_steps(snap[0].cpu().numpy(), snap[1].cpu().numpy(), f0)
        from oracle import oracle as O
        out['cpu_baseline'] = {'value': v, 'unit': 'steps/s', 'cores': O.lib().oracle_num_threads(), 'kind': 'port', 'sample': sample}
    print(json.dumps(out), flush=True)
    sim.close()


ADMM_METRIC = 'steps/s (ADMM-IPC, two cubes, 6k tets)'


def main_admm(args):
    """ADMM-IPC (projects/FastIPC/ADMM_IPC.py, 20 ADMM iterations per step) on the two-cube drop
    of 8^3 hexes per cube (configuration 0's geometry; fixed-corotated, as the script imports):
    W warm-up steps, K timed steps (CUDA events), e2e with the state through pinned host memory;
    the CPU oracle (numpy restatement) on the first ADMM iterations of the same step from the
    same state, scaled to whole steps."""
    from fastipc_gb300 import scenes as SC
    rank = int(os.environ.get('RANK', '0'))
    scene = SC.two_cubes(n=8, seed=0)
    cfg = {'workload': 'ADMM-IPC: two 0.1 m cubes of 8x8x8 hexes x6 tets, upper one rotated (seed 0) and moving at -1 m/s; '
                       'fixed-corotated E=1e5 nu=0.4, dhat=1e-3, dt=0.01, 20 ADMM iterations per step',
           'tets': int(len(scene.tets)), 'verts': int(len(scene.x)), 'pcg_rtol': args.pcg_rtol,
           'l2': 'working set smaller than L2, not flushed between steps (bound by launches and host syncs)'}

    def cpu_sample(x0, v0, f0, iters=2):
        from oracle.admm_oracle import AdmmOracle
        o = AdmmOracle(scene)
        o.x, o.v = x0.copy(), v0.copy()
        t0 = time.perf_counter()
        o.initial_guess()
        for k in range(iters):
            o.admm_iteration(f0, k)
        dt = time.perf_counter() - t0
        return iters / (dt * o.admm_iters), (f'ADMM iterations 0..{iters - 1} of step {f0} of the same scene from the same state '
                                             f'({dt:.1f} s; numpy restatement, one core), scaled to 20 iterations per step')

    if args.impl == 'reference':
        if rank != 0:
            return
        from oracle.admm_oracle import AdmmOracle
        o = AdmmOracle(scene)
        for f in range(args.warmup):
            o.step(f)
        v, sample = cpu_sample(o.x, o.v, args.warmup)
        print(json.dumps({'impl': 'reference', 'metric': ADMM_METRIC, 'value': v, 'unit': 'steps/s', 'n_gpus': args.gpus,
                          'steps': args.steps, 'warmup': args.warmup, 'higher_is_better': True, 'scaling': 'weak',
                          'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'config': cfg,
                          'cpu_baseline': {'value': v, 'unit': 'steps/s', 'cores': 1, 'kind': 'port', 'sample': sample},
                          'e2e': {'value': v, 'unit': 'steps/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}), flush=True)
        return
    import torch
    from fastipc_gb300 import _native
    from fastipc_gb300.admm import AdmmIPC
    from fastipc_gb300.build import build
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    build()
    sim = AdmmIPC(scene, device=dev, pcg_rtol=args.pcg_rtol)
    f = 0
    for _ in range(args.warmup):
        sim.step(f)
        f += 1
    snap = (sim.x.clone(), sim.v.clone())
    f0 = f
    stream = torch.cuda.current_stream(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = _native.launch_count()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            sim.step(f)
            f += 1
        ev1.record(stream)
        torch.cuda.synchronize(dev)
    launches = _native.launch_count() - launches0
    ms = ev0.elapsed_time(ev1)
    hx = torch.empty_like(snap[0], device='cpu').pin_memory()
    hv = torch.empty_like(snap[1], device='cpu').pin_memory()
    hx.copy_(snap[0])
    hv.copy_(snap[1])
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    f = f0
    for _ in range(args.steps):
        sim.x.copy_(hx, non_blocking=True)
        sim.v.copy_(hv, non_blocking=True)
        sim.step(f)
        hx.copy_(sim.x, non_blocking=True)
        hv.copy_(sim.v, non_blocking=True)
        f += 1
    e1.record(stream)
    torch.cuda.synchronize(dev)
    e2e_ms = e0.elapsed_time(e1)
    nbytes = 2 * sim.x.numel() * 8
    its = sim.global_iters[-args.steps * sim.admm_iters:]
    out = {'metric': ADMM_METRIC, 'value': args.steps / (ms / 1e3), 'unit': 'steps/s', 'n_gpus': 1, 'steps': args.steps,
           'warmup': args.warmup, 'ms_per_step': ms / args.steps, 'higher_is_better': True, 'scaling': 'weak',
           'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'config': cfg,
           'ms_per_admm_iter': ms / (args.steps * sim.admm_iters), 'pcg_iters_per_global_step': sum(its) / max(len(its), 1),
           'e2e': {'value': args.steps / (e2e_ms / 1e3), 'unit': 'steps/s', 'h2d_bytes_per_step': nbytes, 'd2h_bytes_per_step': nbytes},
           'gpu_launches': launches, 'clocks': clk.summary()}
    if not args.no_cpu_baseline:
        v, sample = cpu_sample(snap[0].cpu().numpy(), snap[1].cpu().numpy(), f0)
        out['cpu_baseline'] = {'value': v, 'unit': 'steps/s', 'cores': 1, 'kind': 'port', 'sample': sample}
    print(json.dumps(out), flush=True)
    sim.close()


DIRECT_METRIC = 'direct solves/s (216-cube lattice Newton system at first ground contact)'


def main_direct(args):
    """The direct solve of the Newton system (the reference's CHOLMOD role, NEWTON_IPC.py:764-776):
    the 216-cube lattice (configuration 1's scene) stepped with PCG until its first ground
    contact, then its assembled system (elastic and contact blocks) factorised and solved K times
    after W warm-up solves.  A step is one whole direct solve: host analysis, factorisation and
    substitution.  e2e: positions from pinned host memory, assembly, direct solve, direction back.
    The roofline is the factorisation's FP64 flops over the solve time against the measured FP64
    peak.  The CPU arm is the oracle's direct solve (scipy SuperLU) of the same system."""
    from fastipc_gb300 import scenes as SC
    rank = int(os.environ.get('RANK', '0'))
    scene = SC.cube_lattice(m=6, n=6, seed=0)
    cfg = {'workload': 'direct solve of the Newton system of the 6x6x6 lattice of 0.1 m cubes (6 hexes per side x6 tets) on its '
                       'ground box at its first ground contact (PCG steps before it); NH E=1e5 nu=0.4, dhat=1e-3, dt=0.01',
           'tets': int(len(scene.tets)), 'verts': int(len(scene.x)),
           'l2': 'inputs larger than L2 (the fronts hold several GB)'}

    def cpu_solve(x, v, f):
        from oracle import oracle as O
        o = O.OracleSim(scene, solver='direct')
        o.x, o.v = x.copy(), v.copy()
        o.compute_xn_and_xTilde()
        o.move_nodes(f * o.dt)
        o.find_constraints()
        o.compute_hessian_and_gradient()
        t0 = time.perf_counter()
        o.solve_system(f * o.dt)
        dt = time.perf_counter() - t0
        return 1.0 / dt, f'one direct solve of the same system by the oracle (scipy SuperLU, {dt:.1f} s, one core)'

    import numpy as np
    if args.impl == 'reference':
        if rank != 0:
            return
        from oracle import oracle as O
        o = O.OracleSim(scene, solver='bsr', pcg_rtol=1e-8, pcg_maxit=400000)
        f = 0
        while f < 40:
            o.step(f)
            f += 1
            if sum(len(r) for r in o.rows) > 0:
                break
        v, sample = cpu_solve(o.x, o.v, f)
        print(json.dumps({'impl': 'reference', 'metric': DIRECT_METRIC, 'value': v, 'unit': 'solves/s', 'n_gpus': args.gpus,
                          'steps': args.steps, 'warmup': args.warmup, 'higher_is_better': True, 'scaling': 'weak',
                          'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'config': cfg,
                          'cpu_baseline': {'value': v, 'unit': 'solves/s', 'cores': 1, 'kind': 'port', 'sample': sample},
                          'e2e': {'value': v, 'unit': 'solves/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}), flush=True)
        return
    import torch
    from fastipc_gb300 import _native
    from fastipc_gb300.build import build
    from fastipc_gb300.newton import NewtonIPC
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    build()
    sim = NewtonIPC(scene, device=dev, pcg_rtol=1e-8)
    f = 0
    while f < 40:
        sim.step(f)
        f += 1
        if sum(sim.counts) > 0:
            break
    x_h, v_h = sim.x.cpu().numpy().copy(), sim.v.cpu().numpy().copy()
    t = f * sim.dt
    sim.compute_xn_and_xTilde()
    sim.move_nodes(t)
    sim.find_constraints()
    sim.compute_hessian_and_gradient()
    sim.solver = 'direct'
    for _ in range(args.warmup):
        sim.solve_system(t)
    stream = torch.cuda.current_stream(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = _native.launch_count()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            sim.solve_system(t)
        ev1.record(stream)
        torch.cuda.synchronize(dev)
    launches = _native.launch_count() - launches0
    ms = ev0.elapsed_time(ev1) / args.steps
    st = sim.direct_stats()
    p_dir = sim.data_sol.clone()
    sim.solver = 'pcg'
    sim.pcg_rtol, sim.pcg_maxit = 1e-12, 200000
    sim.solve_system(t)
    agree = float(((p_dir - sim.data_sol).abs().max() / sim.data_sol.abs().max()).item())
    sim.solver = 'direct'
    # e2e: state from pinned host memory, assembly, direct solve, direction back to the host
    xs = sim.x.clone()
    hx = torch.empty_like(xs, device='cpu').pin_memory()
    hx.copy_(xs)
    hp = torch.empty_like(sim.data_sol, device='cpu').pin_memory()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        sim.x.copy_(hx, non_blocking=True)
        sim.find_constraints()
        sim.compute_hessian_and_gradient()
        sim.solve_system(t)
        hp.copy_(sim.data_sol, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    e2e_ms = e0.elapsed_time(e1) / args.steps
    pk = fp64_peak(dev)
    achieved = st['flops'] / (ms * 1e-3) / 1e12
    line = {'metric': DIRECT_METRIC, 'value': 1e3 / ms, 'unit': 'solves/s', 'n_gpus': args.gpus, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f64', 'data': 'synthetic', 'config': cfg, 'gpu_launches': int(launches),
            'direct': {'fronts': st['fronts'], 'front_gb': st['front_doubles'] * 8e-9, 'factor_flops': st['flops'],
                       'analyse_ms': st['analyse_ms'], 'contact_rows': int(sum(sim.counts)), 'step_of_first_contact': f,
                       'agreement_with_pcg_1e-12': agree},
            'roofline': {'kernel': 'whole direct solve (k_mf_update holds nearly all its flops)', 'bound': 'fp64',
                         'achieved': achieved, 'peak': pk['tflops'], 'unit': 'TFLOP/s', 'frac': achieved / pk['tflops'],
                         'traffic': None, 'peak_source': 'measured: ' + pk['how'],
                         'note': 'dense factorisation flops of the fronts over the whole solve time (host analysis and '
                                 'substitution included)'},
            'clocks': clk.summary(),
            'e2e': {'value': 1e3 / e2e_ms, 'unit': 'solves/s', 'h2d_bytes_per_step': int(hx.numel() * 8),
                    'd2h_bytes_per_step': int(hp.numel() * 8)}}
    if not args.no_cpu_baseline and rank == 0:
        v, sample = cpu_solve(x_h, v_h, f)
        line['cpu_baseline'] = {'value': v, 'unit': 'solves/s', 'cores': 1, 'kind': 'port', 'sample': sample}
    sim.close()
    _ = np
    if rank == 0:
        print(json.dumps(line), flush=True)


def batch_cpu(scs, args, budget_s=20.0):
    """The oracle steps scenes of the batch (every 16th, after the same warm-up) one at a time
    on the host cores until about budget_s of stepping; scene-steps/s of that sample."""
    from oracle import oracle as O
    done, t_total, names = 0, 0.0, []
    for k in range(0, len(scs), 16):
        sim = O.OracleSim(scs[k], solver='bsr', pcg_rtol=args.pcg_rtol, pcg_maxit=args.cpu_sample_pcg)
        for f in range(args.warmup):
            sim.step(f)
        t0 = time.perf_counter()
        sim.step(args.warmup)
        t_total += time.perf_counter() - t0
        done += 1
        names.append(k)
        if t_total > budget_s:
            break
    sample = f'one time step (step {args.warmup}) of scenes {names} stepped one at a time, {t_total:.1f} s'
    return done / t_total, sample, O.lib().oracle_num_threads()


def learned_leg(sim, snap, f0, args):
    """Newton iterations per step from the timed state with the plain (reference), inertial and
    learned starts, the same steps each (outside the timed value).  The network was trained on
    another jitter seed of the same bar."""
    from fastipc_gb300.learned import LearnedStart, WarmStartMLP, compare_starts
    if not os.path.exists(args.learned_weights):
        return {'unavailable': f'no weights at {os.path.relpath(args.learned_weights, HERE)}'}
    model = WarmStartMLP.load(args.learned_weights, device=sim.device)
    restore(sim, snap)
    warm = sim.pcg_warm_start
    sim.pcg_warm_start = False
    modes = {'plain': None, 'inertial': LearnedStart(kind='inertial'), 'learned': LearnedStart(model, kind='mlp', smooth=4)}
    r = compare_starts(sim, args.learned_steps, f0, modes, log=None)
    sim.pcg_warm_start = warm
    out = {'steps': args.learned_steps, 'first_step': f0, 'weights': os.path.relpath(args.learned_weights, HERE)}
    for k, v in r.items():
        out[k] = {'newton_iters_per_step': v['newton'] / v['steps'], 'steps_per_s': v['steps'] / v['wall_s'],
                  'pcg_iters': v['pcg'], 'intersecting_steps': v['intersecting_steps'], 'chosen': v.get('chosen')}
    out['newton_reduction_vs_inertial'] = 1.0 - r['learned']['newton'] / max(r['inertial']['newton'], 1)
    out['newton_reduction_vs_plain'] = 1.0 - r['learned']['newton'] / max(r['plain']['newton'], 1)
    return out


def ctypes_read(L):
    import ctypes
    t, n, b, fl = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double(), ctypes.c_double()
    L.fipc_profile_read(ctypes.byref(t), ctypes.byref(n), ctypes.byref(b), ctypes.byref(fl))
    return t.value, n.value, b.value, fl.value


if __name__ == '__main__':
    main()
