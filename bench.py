"""Benchmark: FDTD throughput (Mcells/s) of the GB300 solver core on the dispersive-soil model.

Workload (the configuration the headline metric is quoted on): a 400 x 400 x 200 grid at
2 mm, air above z = 150 cells and a 50-material single-pole Debye soil below, binned from a
seeded fractal field, with a buried PEC cylinder, a 10-cell CFS PML on all faces, an
x-polarised Hertzian dipole and a receiver 10 mm above the surface; Ricker 1.5 GHz, fp32
fields, the Debye pole state kept as its fp32 real parts on the device (its imaginary parts are
exactly zero throughout). Synthetic, seeded inputs; no external data.

Metric: Mcells/s = nx*ny*nz*steps / t / 1e6 (the reference's definition; t covers the time
loop only). A step is one full Yee iteration (H half-step, E half-step with the dispersive
update, PML, sources, receiver store).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line. The device-timed ``value`` uses CUDA events on the solver's stream
around K steps (inputs resident; the working set, about 2.5 GB, is far larger than L2).
``e2e`` is the same metric through the public API with host buffers: model upload to the
GPU, K steps and the read-back of the receiver traces inside the timed region.
``roofline`` is for the dominant kernel (the E half-step) from per-launch CUDA events.
``cpu_baseline`` times the reference's own compiled CPU kernels (``oracle/_ref``) on all host
cores on a bounded sample of the same workload (the oracle's C port when those are absent).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, 'oracle'))

METRIC = 'Mcells/s'
WORKLOAD = 'dispersive_soil_400x400x200_debye50_pml10'
# ncu summaries of the E half-step on the soil workload: the full-size capture's
# `dram_bytes_per_launch:` line (dram__bytes_read.sum + dram__bytes_write.sum of one launch of
# the 400x400x200 workload), else the small capture's `dram_bytes_per_cell:` line scaled by cells
TRAFFIC_FULL = os.path.join(ROOT, 'profiles', 'half_step_traffic_dispersive_soil_400x400x200.md')
TRAFFIC_PROFILE = os.path.join(ROOT, 'profiles', 'e_half_step_dispersive_soil_256x256x128.md')
STAGED_TRAFFIC_FULL = os.path.join(ROOT, 'profiles', 'e_half_step_staged_traffic_dispersive_soil_400x400x200.md')
STAGED_TRAFFIC_PROFILE = os.path.join(ROOT, 'profiles', 'e_half_step_staged_dispersive_soil_256x256x128.md')
# the same two lines for the fused step kernel
FUSED_TRAFFIC_FULL = os.path.join(ROOT, 'profiles', 'fused_step_traffic_dispersive_soil_400x400x200.md')
FUSED_TRAFFIC_PROFILE = os.path.join(ROOT, 'profiles', 'fused_step_dispersive_soil_256x256x128.md')


def _profile_value(path, key):
    try:
        with open(path) as f:
            for line in f:
                if line.startswith(key + ':'):
                    return float(line.split(':')[1])
    except OSError:
        pass
    return None


def measured_traffic(cells, fused=False, staged=False):
    """DRAM bytes of one launch of the dominant kernel (the fused step, or the E half-step,
    staged or plain) over `cells` cells (ncu), and where they came from."""
    full_path = FUSED_TRAFFIC_FULL if fused else (STAGED_TRAFFIC_FULL if staged else TRAFFIC_FULL)
    small_path = (FUSED_TRAFFIC_PROFILE if fused else
                  (STAGED_TRAFFIC_PROFILE if staged else TRAFFIC_PROFILE))
    full = _profile_value(full_path, 'dram_bytes_per_launch')
    full_cells = _profile_value(full_path, 'cells')
    if full is not None and full_cells == cells:
        return int(full), 'ncu, full-size launch'
    per_cell = _profile_value(small_path, 'dram_bytes_per_cell')
    if per_cell is not None:
        return int(round(per_cell * cells)), 'ncu, 256x256x128 launch scaled by cells'
    return None, None


def load_peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            p = json.load(f)
        return float(p['hbm_gbs']), 'measured'
    except Exception:
        return 6800.0, 'fallback'


def slab_cells(G):
    """Cells covered by each PML slab (a cell in k slabs counts k times)."""
    n = 0
    for p in G.pmls:
        n += p.nx * p.ny * p.nz
    return n


def algorithmic_bytes(G):
    """Bytes per launch each half-step must move, in the device representation: fp32 fields,
    the node's three material IDs packed in one 32-bit word (nmat <= 1024; otherwise three
    uint32 IDs), complex64 (or real fp32) dispersive state. Per node: H half-step reads E and H and the ID word
    and writes H (12 + 12 + 4 + 12 = 40 B; 36 B when every material has the same H row and no
    ID is needed); E half-step the same (40 B) plus, on nodes whose
    materials have poles, 8 B per pole and component read and written (48 B per pole; 24 B when
    only the real parts are kept, every pole being Debye-like). PML adds
    per slab node and CFS order two Phi values read and written (16 B) in each half-step.
    Neighbour values along j, k and x are re-reads of the same arrays (cache hits)."""
    cells = G.nx * G.ny * G.nz
    idb = 4 if len(G.materials) <= 1024 else 12
    order = max(len(G.cfs), 1)
    pml = slab_cells(G) * 16 * order
    # the H half-step reads no IDs when every material has the same H row (no magnetic ones)
    hrows = np.asarray(G.updatecoeffsH)
    uniform_h = bool((hrows.view(np.uint32) == hrows[:1].view(np.uint32)).all())
    h = cells * (36 + (0 if uniform_h else idb)) + pml
    e = cells * (36 + idb) + pml
    if G.maxpoles:
        disp = np.zeros(len(G.materials), dtype=bool)
        d = np.asarray(G.updatecoeffsdispersive)
        disp[:] = np.any(d != 0, axis=1)
        ids = G.ID[:3, :G.nx, :G.ny, :G.nz]
        dcells = int(np.count_nonzero(disp[ids[0]] | disp[ids[1]] | disp[ids[2]]))
        # complex64 state read and written (48 B per pole), or its real parts only (24 B) when
        # every pole is Debye-like and the device keeps just those
        from gprmax_gb300.solver import real_dispersive_state
        e += dcells * (24 if real_dispersive_state(G) else 48) * G.maxpoles
    return h, e


def fused_bytes(G):
    """Bytes per launch of the fused step (both half-steps in one pass): E and H read once and
    written once (48 B per node), the packed E ID word (4 B) and, unless every material has the
    same H row, the H ID word (4 B); the dispersive state and the E and H PML state as in the
    half-steps. The halo rows, columns and planes the tiles re-read are not counted (they are
    meant to be cache hits)."""
    h, e = algorithmic_bytes(G)
    cells = G.nx * G.ny * G.nz
    # h = cells*(36 [+ id]) + pml, e = cells*40 + pml + disp: the fused step drops one read of
    # E (12 B) and one of H (12 B) per node against their sum
    return h + e - 24 * cells


class ClockSampler:
    """nvidia-smi clock/throttle samples taken while the timed region runs."""

    QUERY = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
             'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
             'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, device=0):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.device), '--query-gpu=' + self.QUERY,
                 '--format=csv,noheader,nounits', '-lms', '100'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(',')])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unsampled'], 'samples': 0}
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace('.', '').isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = set()
        for r in self.rows:
            if len(r) > 8:
                for n, v in zip(names, r[5:9]):
                    if v.lower() == 'active':
                        reasons.add(n)
        return {'sm_mhz': float(np.median(sm)) if sm else None,
                'sm_max_mhz': max(mx) if mx else None,
                'reasons': sorted(reasons), 'samples': len(self.rows)}


def build_workload(iterations, grid=None, snapshot_at=0, pml='10'):
    from gprmax_gb300 import workloads
    if grid:
        nx, ny, nz = grid
        G = workloads.dispersive_soil(nx=nx, ny=ny, nz=nz, surface=int(nz * 0.75),
                                      snapshot_at=snapshot_at, pml=pml)
    else:
        G = workloads.dispersive_soil(snapshot_at=snapshot_at, pml=pml)
    if iterations > G.iterations:
        # longer time window; per-step work is unchanged
        G.iterations = iterations
        for src in G.hertziandipoles + G.voltagesources + G.magneticdipoles:
            src.stop = (iterations - 1) * G.dt
            src.calculate_waveform_values(G)
        for r in G.rxs:
            for k in r.outputs:
                r.outputs[k] = np.zeros(iterations, dtype=np.float32)
    return G


def workload_config(G, args, world):
    """The ``config`` both arms print for the soil workload (the same dict for the same model)."""
    return {'workload': WORKLOAD if not args.grid else 'dispersive_soil_{}x{}x{}'.format(*args.grid),
            'grid': [G.nx, G.ny, G.nz], 'dx_m': G.dx, 'materials': len(G.materials),
            'poles': G.maxpoles,
            'pml_cells': int(args.pml) if len(args.pml.split()) == 1 else [int(v) for v in args.pml.split()],
            'cells': G.nx * G.ny * G.nz,
            'l2': 'working set {:.2f} GB > L2 (129 MB), no flush'.format(dm_bytes(G) / 1e9),
            'replicas': world}


def cpu_model():
    """The host CPU's model name (``/proc/cpuinfo``; the architecture when it names none)."""
    import platform
    part = None
    try:
        with open('/proc/cpuinfo') as f:
            for line in f:
                key = line.split(':')[0].strip().lower()
                if key in ('model name', 'hardware', 'cpu model'):
                    return line.split(':', 1)[1].strip()
                if key == 'cpu part' and part is None:
                    part = line.split(':', 1)[1].strip()
    except OSError:
        pass
    if part:   # Arm cores name themselves by part number only (0xd4f: Neoverse V2, as in Grace)
        return {'0xd4f': 'Arm Neoverse V2'}.get(part.lower(), 'Arm CPU part ' + part)
    return platform.machine()


def cpu_baseline(G, budget_s=20.0, max_steps=60):
    """Bounded CPU run of the same model: reference kernels on all host cores, one warm-up
    step and then at most ``max_steps`` (the model must have ``max_steps + 1`` iterations)."""
    import ref_cpu
    cores = os.cpu_count() or 1
    solver, kind = ref_cpu.make_solver(G, cores)
    t0 = time.perf_counter()
    solver.step()
    t1 = time.perf_counter()
    per = max(t1 - t0, 1e-3)
    n = int(max(2, min(max_steps, budget_s / per)))
    t0 = time.perf_counter()
    for _ in range(n):
        solver.step()
    t = time.perf_counter() - t0
    cells = G.nx * G.ny * G.nz
    return {'value': cells * n / t / 1e6, 'unit': METRIC, 'cores': cores, 'kind': kind,
            'cpu': cpu_model(), 'sample': '{} steps (after 1 warm-up step) of the full {}x{}x{} model, {} OpenMP '
                      'threads'.format(n, G.nx, G.ny, G.nz, cores)}


def dist_setup(n_gpus):
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group('nccl')
    return world, rank, local, dist


def barrier_max(dist, value):
    """The largest `value` over the ranks (the slowest rank's time); the all-reduce is also the
    barrier that closes the timed region."""
    if dist is None:
        return value
    import torch
    device = 'cuda' if dist.get_backend() == 'nccl' else 'cpu'
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world, cells, steps, seconds):
    """Whole-job Mcells/s of `world` replicas, each advancing `cells` cells `steps` steps, when
    the slowest took `seconds` (weak scaling: the work per GPU is fixed)."""
    return world * cells * steps / seconds / 1e6


def run_gb300(args):
    world, rank, local, dist = dist_setup(args.gpus)
    from gprmax_gb300 import _native
    from gprmax_gb300.solver import DeviceModel
    _native.lib()
    K, W = args.steps, args.warmup
    G = build_workload(max(3117, K + W + args.profile_steps + 1), args.grid, args.snapshot_at,
                       args.pml)
    cells = G.nx * G.ny * G.nz
    # warm the CUDA context with a tiny model (not timed)
    from gprmax_gb300.workloads import freespace_dipole
    if not args.no_warm_context:
        tiny = DeviceModel(freespace_dipole(n=20, timewindow='10', pml=4))
        tiny.run()
        tiny.synchronize()
        tiny.close()

    # --- end to end through the public API: upload from host, K steps, read back traces
    if dist is not None:
        dist.barrier()
    options = ((8 if args.half_steps else 0) | (16 if args.plain_e else 0) |
               (32 if args.fused_buffers else 0))
    # the model's inputs in page-locked host memory before the timed region: the material IDs
    # packed two words per node (a third of the ID array's bytes); the copy itself is timed
    from gprmax_gb300.solver import pack_materials
    packed = pack_materials(G)
    t0 = time.perf_counter()
    dm = DeviceModel(G, options, packed=packed)
    if args.staged:
        dm.set_step_forms(True, True)
    t1 = time.perf_counter()
    dm.run(K)
    dm.synchronize()
    t2 = time.perf_counter()
    rx = dm.receivers()
    t_e2e = time.perf_counter() - t0
    e2e_parts = {'model_upload_s': round(t1 - t0, 4), 'steps_s': round(t2 - t1, 4),
                 'readback_s': round(t0 + t_e2e - t2, 4),
                 'upload_detail_s': {k: round(v, 4) for k, v in dm.timings.items()},
                 'materials_s': round(dm.materials_s, 4)}
    h2d = upload_bytes(G, packed)
    d2h = rx.nbytes
    t_e2e = barrier_max(dist, t_e2e)

    # --- device-timed: warm-up, then K steps between events on the solver stream
    dm.reset()
    dm.run(W)
    dm.synchronize()
    if dist is not None:
        dist.barrier()
    with ClockSampler(local) as clk:
        ms = dm.run_timed(K)
    ms = barrier_max(dist, ms)
    # --- per-kernel launch times for the roofline
    ms_h, ms_e, ms_t = dm.profile(max(args.profile_steps, 1))
    checksum = float(np.abs(dm.receivers()).sum())
    step = dm.step_info()
    dm.close()
    fused = step['fused']
    value = replica_rate(world, cells, K, ms / 1e3)
    bytes_h, bytes_e = algorithmic_bytes(G)
    if fused:
        bytes_e = fused_bytes(G)
    peak, peak_kind = load_peaks()
    npf = max(args.profile_steps, 1)
    t_e = ms_e / npf / 1e3
    t_h = ms_h / npf / 1e3
    achieved = bytes_e / t_e / 1e9
    traffic, traffic_src = measured_traffic(cells, fused, step['staged'])
    if fused:
        kernels = {'fused_step': {'ms': t_e * 1e3, 'bytes': bytes_e, 'GBps': round(achieved, 1),
                                  'tile_rows': step['tj'], 'chunks': step['nch'],
                                  'planes_per_chunk': step['planes'], 'blocks': step['blocks']},
                   'step_ms_profiled': ms_t / npf}
    else:
        kernels = {'h_half_step': {'ms': t_h * 1e3, 'bytes': bytes_h,
                                   'GBps': round(bytes_h / t_h / 1e9, 1), 'staged': step['staged_h']},
                   'e_half_step': {'ms': t_e * 1e3, 'bytes': bytes_e,
                                   'GBps': round(achieved, 1), 'staged': step['staged']},
                   'step_ms_profiled': ms_t / npf}
    if rank != 0:
        return
    out = {
        'metric': METRIC, 'value': round(value, 1), 'unit': METRIC, 'n_gpus': world,
        'steps': K, 'warmup': W, 'ms_per_step': ms / K, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
        'data': 'synthetic (seeded fractal Debye soil)',
        'config': workload_config(G, args, world),
        'e2e': {'value': round(replica_rate(world, cells, K, t_e2e), 1), 'unit': METRIC,
                'h2d_bytes_per_step': int(h2d / K), 'd2h_bytes_per_step': int(d2h / K),
                'what': 'DeviceModel(G) upload from page-locked host memory (material IDs packed '
                        'two words per node before the timed region) + {} steps + receiver '
                        'read-back'.format(K),
                'parts': e2e_parts},
        # per step: the fused step and the end-of-step kernel, or H, E and end-of-step
        'gpu_launches': (2 if fused else 3) * K,
        'roofline': {'bound': 'hbm',
                     'kernel': ('fused_step' if fused else
                                'e_half_step_staged' if step['staged'] else 'e_half_step'),
                     'achieved': round(achieved, 1),
                     'peak': peak, 'unit': 'GB/s', 'frac': round(achieved / peak, 4),
                     'traffic': traffic, 'traffic_source': traffic_src, 'peak_source': peak_kind,
                     'bytes_per_launch': bytes_e, 'ms_per_launch': t_e * 1e3},
        'kernels': kernels,
        'clocks': clk.summary(),
        'checksum_rx_abs_sum': checksum,
    }
    if args.cpu_baseline:
        out['cpu_baseline'] = cpu_baseline(G, budget_s=args.cpu_budget)
    if args.extras and world == 1:
        # after the timed region: the batched 2D B-scan (section "bscan2d"), so that its figures
        # come from the same run as the headline
        try:
            b = measure_bscan2d(60, 3)
            out['extras'] = {'bscan2d': {
                'workload': b['config']['workload'], 'traces_per_s_batched': b['value'],
                'traces_per_s_batched_unshared': b['batched_unshared']['value'],
                'traces_per_s_sequential': b['plain_sequential']['value'],
                'speedup_vs_sequential': b['speedup_vs_plain'],
                'traces_identical': b['traces_identical'],
                'models_sharing_geometry': b['batched']['models_sharing_geometry'],
                'h2d_bytes_per_step': b['e2e']['h2d_bytes_per_step'],
                'gpu_launches': b['gpu_launches']}}
        except Exception as e:   # the headline above stands either way
            out['extras'] = {'bscan2d_error': '{}: {}'.format(type(e).__name__, e)}
        # the gradient workload's cost (section "adjoint"; the finite-difference check is left
        # to --workload adjoint)
        try:
            c = adjoint_cost()
            c['solver'].close()
            out['extras']['adjoint'] = {
                'workload': 'adjoint_200x200x100_grf', 'iterations': c['m'].iterations,
                'forward_s': round(c['t_fwd'], 4), 'gradient_s': round(c['t_grad'], 4),
                'gradient_over_forward': round(c['t_grad'] / c['t_fwd'], 3)}
        except Exception as e:
            out['extras']['adjoint_error'] = '{}: {}'.format(type(e).__name__, e)
    print(json.dumps(out), flush=True)


def dm_bytes(G):
    return G.memory_estimate()


def upload_bytes(G, packed=None, materials=True):
    """Host bytes a model's upload copies to the device: material IDs (two packed words per node
    when ``packed``, else the ID array) and coefficient tables (unless ``materials`` is false:
    a model sharing another's), PML profiles and the sources' waveform tables."""
    ids = sum(w.array.nbytes for w in packed if w is not None) if packed else G.ID.nbytes
    mats = (ids + G.updatecoeffsE.nbytes + G.updatecoeffsH.nbytes
            + (G.updatecoeffsdispersive.nbytes if G.maxpoles else 0)) if materials else 0
    return (mats
            + sum(8 * getattr(p, 'ERA').nbytes for p in G.pmls)
            + len(G.hertziandipoles + G.voltagesources + G.magneticdipoles) * G.iterations * 4)


def run_reference(args):
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    import ref_cpu
    K, W = args.steps, args.warmup
    G = build_workload(3117, args.grid, pml=args.pml)
    cores = os.cpu_count() or 1
    solver, kind = ref_cpu.make_solver(G, cores)
    t0 = time.perf_counter()
    for _ in range(max(W, 1)):
        solver.step()
    per = (time.perf_counter() - t0) / max(W, 1)
    n = K
    note = ''
    if per * K > args.ref_budget:
        n = max(2, int(args.ref_budget / per))
        note = ' (bounded to {} of the {} requested steps to stay within {:.0f} s)'.format(n, K, args.ref_budget)
    t0 = time.perf_counter()
    for _ in range(n):
        solver.step()
    t = time.perf_counter() - t0
    cells = G.nx * G.ny * G.nz
    value = cells * n / t / 1e6
    sample = '{} steps after {} warm-up of the full {}x{}x{} model, {} OpenMP threads{}'.format(
        n, max(W, 1), G.nx, G.ny, G.nz, cores, note)
    out = {'metric': METRIC, 'value': round(value, 2), 'unit': METRIC, 'n_gpus': world,
           'steps': n, 'warmup': max(W, 1), 'ms_per_step': t / n * 1e3, 'higher_is_better': True,
           'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
           'data': 'synthetic (seeded fractal Debye soil)', 'impl': 'reference',
           'config': workload_config(G, args, world),
           'cpu_baseline': {'value': round(value, 2), 'unit': METRIC, 'cores': cores,
                            'kind': kind, 'cpu': cpu_model(), 'sample': sample},
           'e2e': {'value': round(value, 2), 'unit': METRIC, 'h2d_bytes_per_step': 0,
                   'd2h_bytes_per_step': 0},
           'gpu_launches': 0}
    print(json.dumps(out), flush=True)


def run_bscan(args):
    """Uneven B-scan: half the models 200x200x100, half 300x300x150 cells at 2 mm, each with
    its own 3-layer soil and buried PEC sphere, the dipole/receiver pair moved 4 mm per model;
    10 ns (2598 iterations). The batched form (one persistent launch per half-step over every
    model, the time loop replayed from one CUDA graph) against the same models run one after
    another through the plain solver. Both arms upload every model from host memory, advance
    it K steps and read its receiver trace back; traces/s scales the K-step times to the full
    2598 iterations (the per-step work does not change with the step index). The host model
    build (input parsing and material-ID build, identical for both arms) is timed separately.
    ``--shapes`` replaces the two model shapes (many small models: the case batching is for)."""
    from gprmax_gb300 import workloads
    from gprmax_gb300.solver import BatchModel, DeviceModel
    K, W = args.steps, args.warmup
    shapes = tuple(tuple(int(v) for v in s.split('x')) for s in args.shapes)
    # the same 128 models built with their geometry in device memory (timed, then freed)
    t0 = time.perf_counter()
    dgrids = workloads.bscan_models(args.models, shapes, device_build=True)
    t_build_dev = time.perf_counter() - t0
    for G in dgrids:
        G.geom.close()
    del dgrids
    t0 = time.perf_counter()
    grids = workloads.bscan_models(args.models, shapes)
    t_build = time.perf_counter() - t0
    iters = min(G.iterations for G in grids)
    cells = sum(G.nx * G.ny * G.nz for G in grids)
    # sequential plain runs: upload, K steps, trace read-back, free, model after model
    warm = DeviceModel(grids[0])
    warm.run(W)
    warm.synchronize()
    warm.close()
    t0 = time.perf_counter()
    dev_plain = 0.0
    for G in grids:
        dm = DeviceModel(G)
        dev_plain += dm.run_timed(K)
        dm.receivers()
        dm.close()
    wall_plain = time.perf_counter() - t0
    upload_plain = wall_plain - dev_plain / 1e3
    # batched: all models resident, one launch per half-step, the K steps as one graph
    t0 = time.perf_counter()
    bm = BatchModel(grids)
    t_up = time.perf_counter() - t0
    bm.run(W)
    bm.synchronize()
    dev_batch = bm.run_timed(K)
    t1 = time.perf_counter()
    bm.receivers()
    t_down = time.perf_counter() - t1
    bm.close()
    # full-length traces: the K-step device time scaled to all iterations plus the per-model
    # upload and read-back costs measured above
    full_plain = upload_plain + dev_plain / 1e3 * iters / K
    full_batch = t_up + t_down + dev_batch / 1e3 * (iters - 0) / K
    out = {'metric': 'traces/s', 'value': round(len(grids) / full_batch, 4), 'unit': 'traces/s',
           'n_gpus': 1, 'steps': K, 'warmup': W, 'ms_per_step': dev_batch / K,
           'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
           'data': 'synthetic (seeded 3-layer soils with buried PEC spheres)',
           'config': {'workload': 'bscan_uneven_{}_models'.format(len(grids)),
                      'shapes': [list(s) for s in shapes], 'iterations': iters,
                      'cells_total': cells},
           'plain_sequential': {'value': round(len(grids) / full_plain, 4), 'unit': 'traces/s',
                                'ms_per_step_all_models': dev_plain / K,
                                'upload_and_readback_s': round(upload_plain, 3)},
           'batched': {'ms_per_step_all_models': dev_batch / K, 'upload_s': round(t_up, 3),
                       'readback_s': round(t_down, 3),
                       'Mcells_per_s': round(cells * K / (dev_batch / 1e3) / 1e6, 1)},
           'speedup_vs_plain': round(full_plain / full_batch, 3),
           'host_build_s': round(t_build, 2), 'device_build_s': round(t_build_dev, 2)}
    print(json.dumps(out), flush=True)


def run_bscan2d(args):
    """2D B-scan: see measure_bscan2d; prints its JSON line."""
    print(json.dumps(measure_bscan2d(args.traces, args.warmup, args.cpu_baseline,
                                     args.cpu_budget)), flush=True)


def measure_bscan2d(ntraces, W, with_cpu=False, cpu_budget=20.0):
    """2D B-scan (``workloads.bscan_2d_models``: TMz, 120x105 cells at 2 mm, a dielectric
    half-space with a buried PEC cylinder, 637 iterations, ``--traces`` traces with the antenna
    pair stepped one cell per trace). Every trace runs to its last iteration in both arms, with
    the upload of each model from host memory and the read-back of its trace inside the timed
    region (wall clock around the public API): the batched form (one launch per half-step over
    every trace, the time loop replayed from one CUDA graph) against the traces run one after
    another through the plain solver. Median of three runs of each arm after a warm-up of each.
    The whole B-scan's state (about 2 MB per trace) stays in L2, as in any run of this model, so
    no flush is done. The host model build (the same for both arms) is timed separately; the
    reference's own kernels on the host cores time one trace."""
    from gprmax_gb300 import workloads
    from gprmax_gb300.solver import BatchModel, DeviceModel
    t0 = time.perf_counter()
    grids = workloads.bscan_2d_models(ntraces)
    t_build = time.perf_counter() - t0
    n = len(grids)
    iters = grids[0].iterations
    cells = grids[0].nx * grids[0].ny * grids[0].nz
    warm = DeviceModel(grids[0])
    warm.run(W)
    warm.synchronize()
    warm.close()
    warm = BatchModel(grids[:2])
    warm.run(W)
    warm.synchronize()
    warm.close()

    def plain():
        t0 = time.perf_counter()
        dev, setup, traces = 0.0, 0.0, []
        for G in grids:
            t1 = time.perf_counter()
            dm = DeviceModel(G)
            setup += time.perf_counter() - t1
            dev += dm.run_timed(iters)
            traces.append(dm.receivers())
            dm.close()
        return time.perf_counter() - t0, dev, traces, setup

    grid_info = {}

    shared_models = []

    def batched(share=True):
        t0 = time.perf_counter()
        bm = BatchModel(grids, share_geometry=share)
        setup = time.perf_counter() - t0
        dev = bm.run_timed(iters)
        traces = bm.receivers()
        if share:
            grid_info.update(bm.info())
            shared_models[:] = [m.shared_from is not None for m in bm.models]
        bm.close()
        return time.perf_counter() - t0, dev, traces, setup

    runs_p = [plain() for _ in range(3)]
    runs_u = [batched(False) for _ in range(3)]
    runs_b = [batched() for _ in range(3)]
    identical = all(np.array_equal(a, b) and np.array_equal(a, c)
                    for a, b, c in zip(runs_p[0][2], runs_b[0][2], runs_u[0][2]))
    wall_p = float(np.median([r[0] for r in runs_p]))
    dev_p = float(np.median([r[1] for r in runs_p]))
    wall_b = float(np.median([r[0] for r in runs_b]))
    dev_b = float(np.median([r[1] for r in runs_b]))
    setup_p = float(np.median([r[3] for r in runs_p]))
    setup_b = float(np.median([r[3] for r in runs_b]))
    wall_u = float(np.median([r[0] for r in runs_u]))
    setup_u = float(np.median([r[3] for r in runs_u]))
    h2d_b = sum(upload_bytes(G, materials=not sh) for G, sh in zip(grids, shared_models))
    rx_bytes = sum(int(np.asarray(t).nbytes) for t in runs_b[0][2])
    out = {'metric': 'traces/s', 'value': round(n / wall_b, 2), 'unit': 'traces/s',
           'n_gpus': 1, 'steps': iters, 'warmup': W, 'ms_per_step': dev_b / iters,
           'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
           'data': 'synthetic (seeded half-space with a buried PEC cylinder)',
           'config': {'workload': 'bscan_2d_cylinder_{}_traces'.format(n),
                      'shape': [grids[0].nx, grids[0].ny, grids[0].nz], 'iterations': iters,
                      'cells_per_trace': cells,
                      'l2': 'no flush: the B-scan state fits in L2 in any run of this model'},
           'e2e': {'value': round(n / wall_b, 2), 'unit': 'traces/s',
                   'h2d_bytes_per_step': round(h2d_b / iters, 1),
                   'd2h_bytes_per_step': round(rx_bytes / iters, 1),
                   'note': 'whole B-scan per timed run: every model uploaded, run and read back'},
           'plain_sequential': {'value': round(n / wall_p, 2), 'unit': 'traces/s',
                                'device_ms_all_traces': round(dev_p, 3),
                                'model_setup_s': round(setup_p, 4)},
           'batched': {'device_ms_all_traces': round(dev_b, 3),
                       'model_setup_s': round(setup_b, 4), 'grid': dict(grid_info),
                       'Mcells_per_s': round(cells * n * iters / (dev_b / 1e3) / 1e6, 1),
                       'models_sharing_geometry': int(sum(shared_models))},
           'batched_unshared': {'value': round(n / wall_u, 2), 'unit': 'traces/s',
                                'model_setup_s': round(setup_u, 4),
                                'h2d_bytes_per_step': round(sum(upload_bytes(G) for G in grids) / iters, 1)},
           'speedup_vs_plain': round(wall_p / wall_b, 3),
           'traces_identical': bool(identical),
           # per batched B-scan: H, E and end-of-step kernels per iteration, and per uploaded
           # geometry one kernel that packs and checks its IDs
           'gpu_launches': 3 * iters + n - int(sum(shared_models)),
           'host_build_s': round(t_build, 3)}
    if with_cpu:
        cb = cpu_baseline(grids[0], budget_s=min(cpu_budget, 20.0), max_steps=iters - 1)
        cb['value'] = round(cb['value'] * 1e6 / (cells * iters), 2)
        cb['unit'] = 'traces/s'
        cb['sample'] = 'one trace, ' + cb['sample']
        out['cpu_baseline'] = cb
    return out


def adjoint_cost(warmup=3):
    """The gradient workload (run_adjoint) timed: the forward (traces and misfit) and the
    gradient (forward with checkpoints, then the adjoint), medians of three after warm-up.
    Returns the model, solver, parameters, observed traces, gradient and times."""
    import torch
    from gprmax_gb300 import workloads
    from gprmax_gb300.adjoint import AdjointModel, AdjointSolver, fdtd_traces
    lines, eps, sig, true = workloads.adjoint_problem()
    m = AdjointModel(lines)
    solver = AdjointSolver(m)
    dev = torch.device('cuda')
    e = torch.tensor(eps, dtype=torch.float64, device=dev)
    s = torch.tensor(sig, dtype=torch.float64, device=dev)
    CAo, CBo = m.edge_coefficients(torch.tensor(true, dtype=torch.float64, device=dev), s)
    obs = solver.forward(CAo.float().contiguous(), CBo.float().contiguous()).double()

    def loss_of(ee):
        CA, CB = m.edge_coefficients(ee, s)
        tr = solver.forward(CA.float().contiguous(), CB.float().contiguous())
        return float(0.5 * ((tr.double() - obs) ** 2).sum())
    for _ in range(max(warmup - 2, 1)):
        loss_of(e)
    fwd_times = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        loss_of(e)
        torch.cuda.synchronize()
        fwd_times.append(time.perf_counter() - t0)
    # the gradient once untimed, then the median of three
    grad_times = []
    for rep in range(4):
        ee = e.clone().requires_grad_(True)
        ss = s.clone().requires_grad_(True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        CA, CB = m.edge_coefficients(ee, ss)
        tr = fdtd_traces(CA, CB, solver)
        L = 0.5 * ((tr.double() - obs) ** 2).sum()
        L.backward()
        torch.cuda.synchronize()
        grad_times.append(time.perf_counter() - t0)
    return {'m': m, 'solver': solver, 'e': e, 's': s, 'obs': obs, 'g': ee.grad, 'eps': eps,
            'loss_of': loss_of, 't_fwd': float(np.median(fwd_times)),
            't_grad': float(np.median(grad_times[1:])), 'fwd_times': fwd_times,
            'grad_times': grad_times, 'misfit': float(L.detach())}


def run_adjoint(args):
    """Gradient of a trace misfit with respect to per-cell eps_r and sigma on a 200x200x100 grid
    at 2 mm, 8 ns (2079 iterations): GRF permittivity, random conductivity, 4 dipoles and 8
    receivers, observed data from a model with a buried 40 mm box 5 % denser. Times the forward
    (traces) and the checkpointed adjoint (gradient), and checks the gradient against central
    finite differences of the same GPU forward (fp64 misfit) on 20 seeded cells among the most
    sensitive 1 %."""
    import torch
    from gprmax_gb300.adjoint import AdjointSolver, fdtd_traces
    cost = adjoint_cost(args.warmup)
    m, solver, e, s = cost['m'], cost['solver'], cost['e'], cost['s']
    obs, g, eps = cost['obs'], cost['g'], cost['eps']
    loss_of, t_fwd, t_grad = cost['loss_of'], cost['t_fwd'], cost['t_grad']
    # finite differences on 20 cells drawn from the 1 % with the largest |gradient|
    flat = g.abs().flatten()
    top = torch.topk(flat, max(20, flat.numel() // 100)).indices.cpu().numpy()
    rng = np.random.default_rng(5)
    cells = rng.choice(top, min(args.fd_cells, top.size), replace=False)
    errs = []
    for c in cells:
        # fourth-order central difference, step 5 % of eps_r (the fp32 forward's rounding noise
        # limits how small the step can be)
        idx = np.unravel_index(int(c), eps.shape)
        h = 0.05 * float(e[idx])
        f = {}
        for k in (-2, -1, 1, 2):
            p = e.clone()
            p[idx] += k * h
            f[k] = loss_of(p)
        fd = (8 * (f[1] - f[-1]) - (f[2] - f[-2])) / (12 * h)
        errs.append(abs(fd - float(g[idx])) / max(abs(fd), 1e-300))
    solver.close()
    # the same gradient with plain sqrt checkpointing (checkpoint_interval 0): a segment every
    # ceil(sqrt(iterations)) steps, all but the last recomputed
    rich = AdjointSolver(m, checkpoint_interval=0)
    rich_times = []
    for rep in range(4):
        ee = e.clone().requires_grad_(True)
        ss = s.clone().requires_grad_(True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        CA, CB = m.edge_coefficients(ee, ss)
        tr = fdtd_traces(CA, CB, rich)
        L2 = 0.5 * ((tr.double() - obs) ** 2).sum()
        L2.backward()
        torch.cuda.synchronize()
        rich_times.append(time.perf_counter() - t0)
    t_rich = float(np.median(rich_times[1:]))
    rich_dev = float((ee.grad - g).abs().max() / g.abs().max())
    rich.close()
    cells_n = m.nx * m.ny * m.nz
    out = {'metric': 'adjoint_over_forward', 'value': round(t_grad / t_fwd, 3), 'unit': 'x',
           'n_gpus': 1, 'steps': m.iterations, 'warmup': args.warmup,
           'ms_per_step': t_fwd / m.iterations * 1e3, 'higher_is_better': False,
           'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32 fields, f64 misfit and gradient',
           'data': 'synthetic (seeded Gaussian random field permittivity)',
           'config': {'workload': 'adjoint_200x200x100_grf', 'grid': [m.nx, m.ny, m.nz],
                      'iterations': m.iterations, 'sources': len(m.sources),
                      'receivers': len(m.receivers)},
           'forward_s': round(t_fwd, 4), 'gradient_s': round(t_grad, 4),
           'gradient_runs_s': [round(t, 4) for t in cost['grad_times']],
           'checkpointing': ('interval -1: the last segment as long as 60 % of the free device '
                             'memory holds (kept from the forward, never recomputed), the steps '
                             'before it in segments of ceil(sqrt(their count))'),
           'sqrt_checkpointing': {'checkpoint_interval': 0, 'gradient_s': round(t_rich, 4),
                                  'adjoint_over_forward': round(t_rich / t_fwd, 3),
                                  'gradient_runs_s': [round(t, 4) for t in rich_times],
                                  'max_rel_diff_vs_default': rich_dev},
           'forward_runs_s': [round(t, 4) for t in cost['fwd_times']],
           'forward_Mcells_per_s': round(cells_n * m.iterations / t_fwd / 1e6, 1),
           'fd_check': {'cells': len(errs), 'stencil': '4th-order central, h = 5 % of eps_r, GPU fp32 forward',
                        'median_rel_err': float(np.median(errs)) if errs else None,
                        'max_rel_err': float(np.max(errs)) if errs else None},
           'misfit': cost['misfit']}
    print(json.dumps(out), flush=True)


def run_sweep(args):
    """Throughput sweep: cubic grids N^3 at 1 mm with a seeded dielectric block in the central
    half and a 10-cell PML, N in {100, ..., 600}. Per N: device-timed Mcells/s of the fused
    kernels, achieved GB/s of the half-steps (algorithmic bytes over the profiled kernel
    times), and the reference's own compiled CPU kernels on all host cores over a bounded
    number of steps."""
    import ref_cpu
    from gprmax_gb300 import workloads
    from gprmax_gb300.solver import DeviceModel
    K, W = args.steps, args.warmup
    rows = []
    peak, peak_kind = load_peaks()
    for n in args.sizes:
        G = workloads.throughput_cube(n)
        cells = G.nx * G.ny * G.nz
        dm = DeviceModel(G)
        dm.run(W)
        dm.synchronize()
        ms = dm.run_timed(K)
        ms_h, ms_e, _ = dm.profile(5)
        dm.close()
        bh, be = algorithmic_bytes(G)
        gbs = (bh + be) / ((ms_h + ms_e) / 5 / 1e3) / 1e9
        row = {'N': n, 'Mcells_per_s': round(cells * K / (ms / 1e3) / 1e6, 1),
               'ms_per_step': ms / K, 'GBps_half_steps': round(gbs, 1),
               'frac_of_peak': round(gbs / peak, 4)}
        if args.cpu_baseline:
            solver, kind = ref_cpu.make_solver(G, os.cpu_count() or 1)
            solver.step()
            t0 = time.perf_counter()
            steps = 0
            while (time.perf_counter() - t0 < args.cpu_budget / len(args.sizes) or steps < 2) \
                    and steps < G.iterations - 2:
                solver.step()
                steps += 1
            t = time.perf_counter() - t0
            row['cpu'] = {'Mcells_per_s': round(cells * steps / t / 1e6, 1), 'steps': steps,
                          'kind': kind, 'cores': os.cpu_count() or 1}
            row['speedup_vs_cpu'] = round(row['Mcells_per_s'] / row['cpu']['Mcells_per_s'], 1)
            del solver
        rows.append(row)
        del G
    out = {'metric': 'Mcells/s', 'value': rows[-1]['Mcells_per_s'], 'unit': 'Mcells/s',
           'n_gpus': 1, 'steps': K, 'warmup': W, 'ms_per_step': rows[-1]['ms_per_step'],
           'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
           'data': 'synthetic (seeded dielectric block)',
           'config': {'workload': 'throughput_sweep_cubes_1mm_pml10', 'sizes': args.sizes,
                      'peak_GBps': peak, 'peak_source': peak_kind},
           'sweep': rows}
    print(json.dumps(out), flush=True)


def run_build(args):
    """Model build (geometry primitives, voxel blocks, per-edge IDs with smoothing, material
    tables, PML coefficients) on the host and in device memory, for the dispersive soil
    (400x400x200, 50 materials, fractal voxel block and a PEC cylinder) and the largest
    throughput cube (a box with smoothing). Wall seconds of ``build_grid`` each way, best of
    ``--steps`` after ``--warmup`` (the device build includes its CUDA work, which every call
    finishes before it returns)."""
    from gprmax_gb300 import workloads
    rows = []
    cases = [('dispersive_soil_400x400x200', lambda dev: workloads.dispersive_soil(device_build=dev)),
             ('throughput_cube_{}'.format(max(args.sizes)),
              lambda dev: workloads.throughput_cube(max(args.sizes), device_build=dev))]
    for name, make in cases:
        row = {'workload': name}
        for dev in (False, True):
            best = None
            for rep in range(args.warmup + args.steps):
                t0 = time.perf_counter()
                G = make(dev)
                t = time.perf_counter() - t0
                if dev:
                    G.geom.close()
                cells = G.nx * G.ny * G.nz
                del G
                if rep >= args.warmup:
                    best = t if best is None else min(best, t)
            row['device_s' if dev else 'host_s'] = round(best, 3)
        row['cells'] = cells
        row['speedup'] = round(row['host_s'] / row['device_s'], 2)
        rows.append(row)
    out = {'metric': 'model build time', 'value': rows[0]['device_s'], 'unit': 's',
           'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup,
           'ms_per_step': rows[0]['device_s'] * 1e3, 'higher_is_better': False,
           'scaling': 'weak', 'vs_baseline': None, 'dtype': 'u32',
           'data': 'synthetic (seeded fractal Debye soil; seeded dielectric block)',
           'config': {'workload': rows[0]['workload'] + ' build'}, 'builds': rows}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__.split('\n')[0])
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=1000)
    ap.add_argument('--warmup', type=int, default=20)
    ap.add_argument('--impl', choices=['gb300', 'reference'], default='gb300')
    ap.add_argument('--profile-steps', type=int, default=50)
    ap.add_argument('--no-cpu-baseline', dest='cpu_baseline', action='store_false')
    ap.add_argument('--cpu-budget', type=float, default=20.0)
    ap.add_argument('--ref-budget', type=float, default=150.0)
    ap.add_argument('--grid', type=int, nargs=3, default=None,
                    help='smaller soil grid (profiling runs); default 400 400 200')
    ap.add_argument('--pml', default='10',
                    help="soil: PML cells, one value or six (x0 y0 z0 xmax ymax zmax), as #pml_cells")
    ap.add_argument('--snapshot-at', type=int, default=0,
                    help='soil: add a snapshot of the whole domain at this iteration (profiling)')
    ap.add_argument('--fd-cells', type=int, default=20,
                    help='adjoint: cells of the finite-difference check (0: none)')
    ap.add_argument('--half-steps', action='store_true',
                    help='soil: step with the two half-step kernels instead of the fused step')
    ap.add_argument('--fused-buffers', action='store_true',
                    help='soil: give the model the fused step\'s second field buffer although it '
                         'has PML slabs (with GBF_FUSED_TILE, to time the fused step there)')
    ap.add_argument('--staged', action='store_true',
                    help='soil: both half-steps as staged sweeps, without the form tuner (for ncu, '
                         'under which the tuner\'s own timings are distorted)')
    ap.add_argument('--plain-e', action='store_true',
                    help='soil: the plain E half-step kernel instead of the staged sweep')
    ap.add_argument('--no-extras', dest='extras', action='store_false',
                    help='soil: skip the 2D B-scan summary added to the line after the timed region')
    ap.add_argument('--no-warm-context', action='store_true',
                    help='skip the small context warm-up model (launch counting for ncu)')
    ap.add_argument('--workload', choices=['soil', 'bscan', 'bscan2d', 'adjoint', 'sweep', 'build'],
                    default='soil',
                    help='soil: the 400x400x200 Debye soil (default); bscan: the batched uneven '
                         'B-scan against sequential plain runs; bscan2d: a whole 2D B-scan, '
                         'batched against sequential; adjoint: gradient cost and '
                         'finite-difference check of the differentiable time loop; sweep: '
                         'cubes of 100^3 to 600^3 cells; build: model build on the host and '
                         'in device memory')
    ap.add_argument('--models', type=int, default=128, help='bscan: number of models')
    ap.add_argument('--traces', type=int, default=60, help='bscan2d: number of traces')
    ap.add_argument('--shapes', nargs=2, default=['200x200x100', '300x300x150'],
                    help='bscan: the two model shapes, NXxNYxNZ cells at 2 mm')
    ap.add_argument('--sizes', type=int, nargs='+', default=[100, 200, 300, 400, 500, 600],
                    help='sweep: cube edge lengths in cells')
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == 'bscan':
        run_bscan(args)
    elif args.workload == 'bscan2d':
        run_bscan2d(args)
    elif args.workload == 'adjoint':
        run_adjoint(args)
    elif args.workload == 'build':
        run_build(args)
    elif args.workload == 'sweep':
        run_sweep(args)
    elif args.impl == 'reference':
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == '__main__':
    main()
