"""Benchmark of the pyfe3d element-assembly path on GB300.

One step = Quad4.update_KC0 (indices + values, += semantics) over every
element of the 1001x1001-node perturbed plate (1,000,000 Quad4 elements,
per-element thickness), with inputs and COO outputs resident in HBM.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Rank 0 prints one JSON line.  ``--impl reference`` times the CPU oracle (the
C restatement of the reference's per-element routines) on the host cores.
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

METRIC = 'Quad4 KC0 elem/s; solves/s at 1e-8 residual, learned-PC vs plain PCG'
KC0_SIZE = 576
# algorithmic bytes per element of update_KC0 (indices + values, +=):
# values read + written, row and column indices written (576 x 8 B each),
# DOF offsets 32 B, init_k 8 B, pid 4 B, property record 224 B, nodal
# coordinates 24 B (one node per element on a structured mesh).
BYTES_PER_ELEM = KC0_SIZE * 8 * 4 + 32 + 8 + 4 + 224 + 24
# DRAM bytes per element measured by ncu on a 90,000-element launch of the
# current kernel (441.6 MB read + 1203.8 MB written)
TRAFFIC_PER_ELEM = (441.575168e6 + 1203.847e6) / 90000


def max_over_ranks(ms, dist=None, device='cpu'):
    """The timed region's length as the slowest rank saw it (every rank gets
    the maximum; a single process keeps its own)."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(ms, steps, units_per_rank_step, world):
    """Per-step time and the whole-job rate: the units all ranks processed in
    one step over the slowest rank's step time."""
    ms_per_step = ms / steps
    return ms_per_step, units_per_rank_step * world / (ms_per_step / 1e3)


def dist_env():
    rank = int(os.environ.get('RANK', 0))
    world = int(os.environ.get('WORLD_SIZE', 1))
    local = int(os.environ.get('LOCAL_RANK', 0))
    return rank, world, local


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,'
             'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
             'clocks_event_reasons.sw_power_cap')
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.index), '--query-gpu=' + q,
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(',')]
            if len(parts) == 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unsampled']}
        sm = [float(s[0]) for s in self.samples if s[0].replace('.', '').isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i] == 'Active'})
        return {'sm_mhz': float(np.median(sm)) if sm else None,
                'sm_max_mhz': max(mx) if mx else None, 'reasons': reasons,
                'samples': len(self.samples)}


def workload(n_nodes):
    from pyfe3d_gb300.meshes import config2
    m, props, pid, bk, f = config2(n_nodes)
    return m, props, pid


def _ref_props(ref, props, pid, lo, hi):
    """ShellProp objects of the reference for elements [lo, hi) (its own
    class, fields set from the same records)."""
    from pyfe3d_gb300.shellprop import SHELL_FIELDS
    out = []
    for e in range(lo, hi):
        rec = props[pid[e]]
        p = ref.ShellProp()
        for i, f in enumerate(SHELL_FIELDS):
            setattr(p, f, float(rec[i]))
        out.append(p)
    return out


_REFW = {}


def _refw_init(nodes):
    """Worker set-up of the reference arm: the compiled reference and the
    same seeded plate."""
    from oracle import build_ref
    ref = build_ref.load()
    if ref is None:
        raise RuntimeError('the compiled reference is missing')
    m, props, pid = workload(nodes)
    _REFW.update(ref=ref, m=m, props=props, pid=pid)


def _refw_run(lo, hi):
    """The reference's own assembly loop (tests/test_quad4_static_point_load.py:
    60-76) over elements [lo, hi): a Quad4 per element, its DOF offsets and
    offset into the KC0 arrays, update_rotation_matrix, update_probe_xe and
    update_KC0 (indices + values); returns (elements, seconds, checksum).
    The ShellProp objects are made before the timed loop."""
    ref, m, props, pid = _REFW['ref'], _REFW['m'], _REFW['props'], _REFW['pid']
    n = hi - lo
    P = _ref_props(ref, props, pid, lo, hi)
    size = ref.Quad4Data().KC0_SPARSE_SIZE
    KC0r = np.zeros(size * n, dtype=ref.INT)
    KC0c = np.zeros(size * n, dtype=ref.INT)
    KC0v = np.zeros(size * n, dtype=ref.DOUBLE)
    x = m.x
    cd = m.cdof
    probe = ref.Quad4Probe()
    t0 = time.perf_counter()
    for i in range(n):
        e = lo + i
        q = ref.Quad4(probe)
        q.c1 = int(cd[e, 0])
        q.c2 = int(cd[e, 1])
        q.c3 = int(cd[e, 2])
        q.c4 = int(cd[e, 3])
        q.init_k_KC0 = size * i
        q.update_rotation_matrix(x)
        q.update_probe_xe(x)
        q.update_KC0(KC0r, KC0c, KC0v, P[i])
    dt = time.perf_counter() - t0
    return n, dt, float(np.abs(KC0v).sum())


class RefPool:
    """The compiled reference on the host cores: the elements of a step are
    split into one contiguous slice per worker process (spawned, no GPU)."""

    def __init__(self, nodes, workers):
        import multiprocessing as mp
        self.workers = workers
        self.pool = mp.get_context('spawn').Pool(workers, initializer=_refw_init, initargs=(nodes,))

    def run(self, lo, hi):
        """The reference over [lo, hi) on all workers at once; the step's time
        is the slowest worker's assembly loop (the property objects each
        worker makes for its slice beforehand are not part of update_KC0)."""
        n = hi - lo
        w = self.workers
        cuts = [lo + (n * k) // w for k in range(w + 1)]
        res = self.pool.starmap(_refw_run, [(cuts[k], cuts[k + 1]) for k in range(w)])
        return n, max(r[1] for r in res), res

    def close(self):
        self.pool.close()
        self.pool.join()


def reference_available():
    try:
        from oracle import build_ref
        return build_ref.load() is not None
    except Exception:  # noqa: BLE001 -- reported as the port fallback
        return False


def cpu_baseline(m, props, pid, seconds=12.0, threads=None, nodes=1001):
    """The reference's own update_KC0 (compiled from its sources) on the
    host cores over a bounded slice of the same plate; the oracle port when
    the compiled reference is missing."""
    if reference_available():
        workers = threads or os.cpu_count() or 1
        pool = RefPool(nodes, workers)
        try:
            pool.run(0, 4 * workers)  # warm the workers
            n = min(m.E, 12000 * workers)
            done, dt, _ = pool.run(0, n)
        finally:
            pool.close()
        out = {'value': done / dt, 'unit': 'elem/s', 'cores': workers, 'kind': 'reference',
               'sample': 'pyfe3d Quad4 update_KC0 loop (update_rotation_matrix, update_probe_xe, '
                         'update_KC0) over the first %d elements of the 1001x1001 plate, one slice per '
                         'process' % n}
        return out
    from oracle import oracle
    oracle.build()
    if threads:
        oracle.set_threads(threads)
    cores = oracle.num_threads()
    n = min(m.E, 20000)
    total = 0
    t0 = time.perf_counter()
    while True:
        ik = KC0_SIZE * np.arange(n, dtype=np.int64)
        oracle.q4_kc0_batch(m.cdof[:n], ik, m.x, props, pid=pid[:n])
        total += n
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    return {'value': total / dt, 'unit': 'elem/s', 'cores': cores, 'kind': 'port',
            'sample': '%d Quad4 update_KC0 calls (first %d elements of the 1001x1001 plate, '
                      'repeated for %.1f s)' % (total, n, dt)}


def run_reference(args, rank, world):
    """The reference's own CPU path on the host cores: the compiled pyfe3d
    update_KC0 loop, all workers, over the same 1001x1001 plate.  The timed
    steps together cover every element once (step i takes the i-th of
    `steps` equal slices); warm-up steps run a small slice."""
    if rank != 0:
        return
    m, props, pid = workload(args.nodes)
    if not reference_available():
        return run_reference_port(args, m, props, pid, world)
    workers = args.ref_workers or os.cpu_count() or 1
    pool = RefPool(args.nodes, workers)
    try:
        for i in range(args.warmup):
            pool.run(0, 64 * workers)
        E = m.E
        total_t, total_n = 0., 0
        for k in range(args.steps):
            lo, hi = (E * k) // args.steps, (E * (k + 1)) // args.steps
            n, dt, _ = pool.run(lo, hi)
            total_t += dt
            total_n += n
    finally:
        pool.close()
    one = None
    try:
        _refw_init(args.nodes)
        n1, t1, _ = _refw_run(0, 3000)
        one = n1 / t1
    except Exception:  # noqa: BLE001 -- optional figure
        pass
    v = total_n / total_t
    sample = ('pyfe3d Quad4 update_KC0 loop (update_rotation_matrix, update_probe_xe, update_KC0, the '
              'reference tests\' assembly loop) over all %d elements of the plate, split into %d steps, '
              'each step one contiguous slice per worker process' % (total_n, args.steps))
    out = {'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': 'elem/s', 'n_gpus': world,
           'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': total_t / args.steps * 1e3,
           'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
           'data': 'synthetic (seeded perturbed plate, log-normal thickness)',
           'config': {'workload': 'quad4_kc0_plate_%dx%d_nodes' % (args.nodes, args.nodes),
                      'elements': m.E, 'sample': sample},
           'cpu_baseline': {'value': v, 'unit': 'elem/s', 'cores': workers, 'kind': 'reference',
                            'sample': sample, 'single_core_elem_per_s': one},
           'e2e': {'value': v, 'unit': 'elem/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(out))


def run_reference_port(args, m, props, pid, world):
    """The C restatement of the reference (oracle port) when the compiled
    reference is missing."""
    steps = []
    for i in range(args.warmup + args.steps):
        res = cpu_baseline(m, props, pid, seconds=args.ref_seconds)
        if i >= args.warmup:
            steps.append(res['value'])
    v = float(np.mean(steps))
    res['value'] = v
    out = {'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': 'elem/s', 'n_gpus': world,
           'steps': args.steps, 'warmup': args.warmup, 'higher_is_better': True,
           'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
           'config': {'workload': 'quad4_kc0_plate_%dx%d_nodes' % (args.nodes, args.nodes),
                      'elements': m.E, 'sample': res['sample']},
           'cpu_baseline': res,
           'e2e': {'value': v, 'unit': 'elem/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(out))


def run_ours(args, rank, world, local):
    import torch
    from pyfe3d_gb300 import _lib, batch
    torch.cuda.set_device(local)
    lib = _lib.load()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl')
    m, props, pid = workload(args.nodes)
    E = m.E
    dev = torch.device('cuda', local)
    x = torch.from_numpy(m.x).to(dev)
    cdof = torch.from_numpy(m.cdof).to(dev)
    init_k = torch.from_numpy(m.init_k(KC0_SIZE)).to(dev)
    P = torch.from_numpy(props).to(dev)
    pidt = torch.from_numpy(pid).to(dev)
    n = KC0_SIZE * E
    Kr = torch.zeros(n, dtype=torch.int64, device=dev)
    Kc = torch.zeros(n, dtype=torch.int64, device=dev)
    Kv = torch.zeros(n, dtype=torch.float64, device=dev)
    err = _lib.err_word()
    stream = torch.cuda.current_stream()

    def step():
        rc = lib.fe3d_quad4_kc0(E, _lib.ptr(cdof), _lib.ptr(init_k), _lib.ptr(x), x.numel(), None, 0,
                                None, None, None, None, _lib.ptr(P), P.shape[0], _lib.ptr(pidt),
                                _lib.ptr(Kr), _lib.ptr(Kc), _lib.ptr(Kv), n, 0, _lib.ptr(err),
                                _lib.c_vp(stream.cuda_stream))
        if rc:
            raise RuntimeError('fe3d_quad4_kc0 failed: %d' % rc)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    _lib.check(0, 'warmup', err)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    barrier()
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        barrier()
    ms = max_over_ranks(ev0.elapsed_time(ev1), dist, dev)
    ms_per_step, value = whole_job_rate(ms, args.steps, E, world)
    _lib.check(0, 'timed', err)

    # streaming bound of the same access mix: read and write the values once,
    # write rows and columns once (PyTorch's elementwise kernels, no element
    # work), the attainable rate for KC0's bytes on this part
    stream_bound = None
    if rank == 0:
        def stream_step():
            Kv.add_(1.0)
            Kr.fill_(1)
            Kc.fill_(2)
        stream_step()
        torch.cuda.synchronize()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        for _ in range(5):
            stream_step()
        s1.record(stream)
        torch.cuda.synchronize()
        sms = s0.elapsed_time(s1) / 5
        sbytes = 4 * 8 * n  # values read + written, rows and columns written
        stream_bound = {'ms': sms, 'gbs': sbytes / (sms / 1e3) / 1e9,
                        'bytes': sbytes, 'kc0_fraction': sms / ms_per_step,
                        'note': 'Kv.add_ + Kr.fill_ + Kc.fill_ over the same arrays'}

    # end to end through the public API with pinned host buffers
    e2e = None
    if rank == 0 and not args.no_e2e:
        e2e = run_e2e(args, m, props, pid)

    if rank != 0:
        return
    with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) if os.path.exists(
            os.path.join(ROOT, 'MEASURED_PEAKS.json')) else open(os.devnull) as fh:
        try:
            peaks = json.load(fh)
        except Exception:
            peaks = {}
    peak = peaks.get('hbm_gbs')
    peak_src = 'measured'
    if not peak:
        peak, peak_src = 6800.0, 'fallback'
    achieved = BYTES_PER_ELEM * E / (ms_per_step / 1e3) / 1e9
    out = {
        'metric': METRIC, 'value': value, 'unit': 'elem/s', 'n_gpus': world, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms_per_step, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
        'dtype_note': ('element matrices in FP64; for elements flat in the XY plane the Jacobian, its inverse '
                       'and the shape-derivative products are float-float (about 48 significant bits, FP32 '
                       'pipe); every element block matches the FP64 oracle to 1e-12 of its largest entry, '
                       'ill-conditioned elements included'),
        'data': 'synthetic (seeded perturbed plate, log-normal thickness)',
        'config': {'workload': 'quad4_kc0_plate_%dx%d_nodes' % (args.nodes, args.nodes),
                   'elements': E, 'dofs': m.N, 'coo_triplets': n,
                   'l2': 'inputs+outputs %.1f GB > L2, no flush needed' % (BYTES_PER_ELEM * E / 1e9),
                   'parallelism': 'replicas' if world > 1 else 'single'},
        'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                     'frac': achieved / peak, 'peak_source': peak_src,
                     'traffic': (args.traffic_per_launch if args.traffic_per_launch is not None
                                 else TRAFFIC_PER_ELEM * E),
                     'traffic_source': 'ncu dram__bytes_read+write of a 90,000-element launch '
                                       'of the same kernel, scaled by the element count',
                     'bytes_per_elem': BYTES_PER_ELEM},
        'stream_bound': stream_bound,
        'clocks': clk.summary(),
        'gpu_launches': args.steps,
    }
    if e2e is not None:
        out['e2e'] = e2e
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(m, props, pid, seconds=args.ref_seconds, nodes=args.nodes)
    # the sections after the headline measurement report their own failure
    # instead of losing the line
    del Kr, Kc, Kv
    torch.cuda.empty_cache()
    for key, skip, fn in (('other_kernels', args.no_other, bench_other_kernels),
                          ('fused_kc0_csr', args.no_fused, bench_fused),
                          ('solve', args.no_solve, bench_solve),
                          ('panel', args.no_panel, bench_panel),
                          ('batched_plates', args.no_batch, bench_batch),
                          ('learned_pc', args.no_learned, bench_learned)):
        if skip:
            continue
        try:
            out[key] = fn(args)
        except Exception as e:  # noqa: BLE001
            out[key] = {'error': '%s: %s' % (type(e).__name__, e)}
            print('bench section %s failed: %r' % (key, e), file=sys.stderr)
    print(json.dumps(out))


def bench_other_kernels(args):
    """The other element kernels on the same plate (one launch each):
    Quad4 KG from a global displacement field, Quad4 M (mtype 0), and BeamC
    KC0 on beams along the plate's node lines.  CUDA events around each."""
    import torch
    from pyfe3d_gb300 import _lib, batch
    from pyfe3d_gb300.meshes import config2, stringer_records
    m, props, pid, bk, f = config2(args.nodes)
    dev = torch.device('cuda')
    E = m.E
    x = torch.from_numpy(m.x).to(dev)
    cdof = torch.from_numpy(m.cdof).to(dev)
    P = torch.from_numpy(props).to(dev)
    pidt = torch.from_numpy(pid).to(dev)
    rng = np.random.default_rng(7)
    u = torch.from_numpy(rng.normal(size=m.N) * 1e-4).to(dev)
    out = {}

    def timed(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    for name, size, fn_make in (
            ('quad4_kg', 144, lambda r, c, v, ik: (lambda: batch.quad4_update_KG(
                r, c, v, x, u, cdof, ik, P, pid=pidt, check=False))),
            ('quad4_m0', 480, lambda r, c, v, ik: (lambda: batch.quad4_update_M(
                r, c, v, x, cdof, ik, P, pid=pidt, mtype=0, check=False)))):
        n = size * E
        r = torch.zeros(n, dtype=torch.int64, device=dev)
        c = torch.zeros(n, dtype=torch.int64, device=dev)
        v = torch.zeros(n, dtype=torch.float64, device=dev)
        ik = torch.from_numpy(m.init_k(size)).to(dev)
        ms = timed(fn_make(r, c, v, ik))
        note = None
        if name == 'quad4_kg':
            # on a plate flat in z only the 16 (w, w) values of the 144 change
            # (the others are += 0 and are not touched); the indices are all written
            nv = 16 if float(np.ptp(m.x[2::3])) == 0. else 144
            nbytes = 144 * 16 + nv * 16 + 32 + 8 + 4 + 224 + 24 + 192
            note = '144 indices + %d values read and written per element, inputs, ue gather' % nv
        else:
            nbytes = size * 32 + 32 + 8 + 4 + 224 + 24
        out[name] = {'ms': ms, 'elem_per_s': E / (ms / 1e3), 'bytes_per_elem': nbytes,
                     'achieved_gbs': nbytes * E / (ms / 1e3) / 1e9}
        if note:
            out[name]['note'] = note
        del r, c, v
        torch.cuda.empty_cache()
    # reduced-integration shells on the same nodes: Quad4R on the quads,
    # Tria3R on each quad split into two triangles
    tcdof_np = np.empty((2 * E, 3), np.int64)
    tcdof_np[0::2] = m.cdof[:, [0, 1, 2]]
    tcdof_np[1::2] = m.cdof[:, [0, 2, 3]]
    tpid_np = np.repeat(pid, 2)
    for name, size, ecdof_np, epid_np, fn in (
            ('quad4r_kc0', 576, m.cdof, pid, batch.quad4r_update_KC0),
            ('tria3r_kc0', 324, tcdof_np, tpid_np, batch.tria3r_update_KC0)):
        En = len(ecdof_np)
        nn = ecdof_np.shape[1]
        ecdof = torch.from_numpy(ecdof_np).to(dev)
        epid = torch.from_numpy(epid_np).to(dev)
        n = size * En
        r = torch.zeros(n, dtype=torch.int64, device=dev)
        c = torch.zeros(n, dtype=torch.int64, device=dev)
        v = torch.zeros(n, dtype=torch.float64, device=dev)
        ik = torch.from_numpy(size * np.arange(En, dtype=np.int64)).to(dev)
        ms = timed(lambda: fn(r, c, v, x, ecdof, ik, P, pid=epid, check=False))
        ms_vo = timed(lambda: fn(r, c, v, x, ecdof, ik, P, pid=epid, update_KC0v_only=1, check=False))
        # rows, columns and values written, values read; offsets, ids,
        # records and coordinates read once
        nbytes = size * 32 + 8 * nn + 8 + 4 + 224 + 24 * nn
        nbytes_vo = size * 16 + 8 * nn + 8 + 4 + 224 + 24 * nn
        out[name] = {'ms': ms, 'elements': int(En), 'elem_per_s': En / (ms / 1e3), 'bytes_per_elem': nbytes,
                     'achieved_gbs': nbytes * En / (ms / 1e3) / 1e9,
                     'values_only': {'ms': ms_vo, 'elem_per_s': En / (ms_vo / 1e3),
                                     'achieved_gbs': nbytes_vo * En / (ms_vo / 1e3) / 1e9}}
        if not args.no_cpu:
            # the oracle (all host threads) on the first 40,000 elements
            from oracle import oracle as orc
            ns = 40000
            ref = orc.t3_kc0_batch if nn == 3 else orc.q4r_kc0_batch
            t0 = time.perf_counter()
            ref(ecdof_np[:ns], size * np.arange(ns, dtype=np.int64), m.x, props, pid=epid_np[:ns])
            dt = time.perf_counter() - t0
            out[name]['cpu_baseline'] = {'elem_per_s': ns / dt, 'kind': 'port', 'cores': orc.num_threads(),
                                         'sample': '%d elements' % ns}
        del r, c, v
        torch.cuda.empty_cache()
    # beams: every node row of the plate as a chain of BeamC elements
    nids = m.nids
    n1 = nids[:-1, :].ravel()
    n2 = nids[1:, :].ravel()
    Eb = n1.size
    bcdof = torch.from_numpy(6 * np.stack([n1, n2], 1).astype(np.int64)).to(dev)
    bprops = torch.from_numpy(stringer_records()[None, :]).to(dev)
    n = 144 * Eb
    r = torch.zeros(n, dtype=torch.int64, device=dev)
    c = torch.zeros(n, dtype=torch.int64, device=dev)
    v = torch.zeros(n, dtype=torch.float64, device=dev)
    ik = torch.from_numpy(144 * np.arange(Eb, dtype=np.int64)).to(dev)
    vxy = torch.tensor([0., 1., 0.], dtype=torch.float64, device=dev)
    ms = timed(lambda: batch.beamc_update_KC0(r, c, v, x, bcdof, ik, vxy, bprops, check=False))
    nbytes = 144 * 32 + 16 + 8 + 128 + 48
    out['beamc_kc0'] = {'ms': ms, 'elem_per_s': Eb / (ms / 1e3), 'elements': int(Eb),
                        'bytes_per_elem': nbytes, 'achieved_gbs': nbytes * Eb / (ms / 1e3) / 1e9,
                        'note': 'frame kernel + matrix kernel (two launches)'}
    # the remaining element updates of the path, timed the same way (elements/s
    # only); each reports its own failure
    ub = torch.from_numpy(rng.normal(size=m.N) * 1e-4).to(dev)
    extra = (
        ('beamc_kg', Eb, lambda: batch.beamc_update_KG(r, c, v, x, ub, bcdof, ik, vxy, bprops, check=False)),
        ('beamc_m0', Eb, lambda: batch.beamc_update_M(r, c, v, x, bcdof, ik, vxy, bprops, mtype=0, check=False)),
    )
    for name, En, fn in extra:
        try:
            ms = timed(fn)
            out[name] = {'ms': ms, 'elem_per_s': En / (ms / 1e3), 'elements': int(En)}
        except Exception as ex:  # noqa: BLE001 -- reported in the line
            out[name] = {'error': repr(ex)[:200]}
    del r, c, v
    torch.cuda.empty_cache()
    try:
        n = 144 * E
        r = torch.zeros(n, dtype=torch.int64, device=dev)
        c = torch.zeros(n, dtype=torch.int64, device=dev)
        v = torch.zeros(n, dtype=torch.float64, device=dev)
        ik = torch.from_numpy(m.init_k(144)).to(dev)
        nstress = torch.from_numpy(rng.normal(size=(E, 3)) * 1e3).to(dev)
        ms = timed(lambda: batch.quad4_update_KG_given_stress(r, c, v, x, cdof, ik, nstress, check=False))
        out['quad4_kg_given_stress'] = {'ms': ms, 'elem_per_s': E / (ms / 1e3), 'elements': int(E)}
        del r, c, v
        torch.cuda.empty_cache()
    except Exception as ex:  # noqa: BLE001 -- reported in the line
        out['quad4_kg_given_stress'] = {'error': repr(ex)[:200]}
    try:
        fint = torch.zeros(m.N, dtype=torch.float64, device=dev)
        ms = timed(lambda: batch.quad4_update_fint(fint, x, u, cdof, P, pid=pidt, check=False))
        out['quad4_fint'] = {'ms': ms, 'elem_per_s': E / (ms / 1e3), 'elements': int(E),
                             'note': 'probe ue + KC0e ue + R turn + atomic scatter into fint'}
    except Exception as ex:  # noqa: BLE001 -- reported in the line
        out['quad4_fint'] = {'error': repr(ex)[:200]}
    return out


def bench_fused(args):
    """KC0 -> reduced CSR per update on the scale plate: the triplet path
    (update_KC0 into COO arrays, then the numeric assembly over the pattern)
    against the fused path (the Quad4 KC0 kernel adding its blocks straight
    into the CSR values through the element -> CSR map, no triplets), with
    the pattern and map set-up times and the largest difference of the two."""
    import torch
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import config2
    from pyfe3d_gb300.solver import CSRPattern, ElementPattern, FusedMap
    m, props, pid, bk, f = config2(args.nodes)
    dev = torch.device('cuda')
    E = m.E
    x = torch.from_numpy(m.x).to(dev)
    cdof = torch.from_numpy(m.cdof).to(dev)
    P = torch.from_numpy(props).to(dev)
    pidt = torch.from_numpy(pid).to(dev)

    def timed(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    t0 = time.perf_counter()
    pat = ElementPattern([cdof], m.N, bk)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    fm = FusedMap(pat, [cdof])
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    vals = fm.new_values()
    out = {'workload': 'quad4_kc0_plate_%dx%d_nodes -> reduced CSR (clamped)' % (args.nodes, args.nodes),
           'elements': E, 'free_dofs': int(pat.nrows), 'nnz': int(pat.nnz),
           'pattern_from_elements_s': t1 - t0, 'map_s': t2 - t1, 'colours': [int(c) for c in fm.colors()]}
    for mode in ('assign', 'atomic'):
        if mode == 'atomic':
            fn = (lambda: (vals.zero_(), batch.quad4_update_KC0_csr(vals, fm, x, P, pid=pidt, mode='atomic',
                                                                     check=False)))
        else:
            fn = (lambda: batch.quad4_update_KC0_csr(vals, fm, x, P, pid=pidt, mode='assign', check=False))
        ms = timed(fn)
        out[mode] = {'ms_per_update': ms, 'elem_per_s': E / (ms / 1e3)}
    out['assign']['note'] = ('one launch per element colour, read-add-write of the CSR entries without atomics '
                             '(deterministic; the first contributor of each block stores)')
    out['atomic']['note'] = 'clearing of the values + one launch with atomic additions (order unspecified)'
    batch.quad4_update_KC0_csr(vals, fm, x, P, pid=pidt)
    # the triplet path on the same plate
    n = KC0_SIZE * E
    Kr = torch.zeros(n, dtype=torch.int64, device=dev)
    Kc = torch.zeros(n, dtype=torch.int64, device=dev)
    Kv = torch.zeros(n, dtype=torch.float64, device=dev)
    ik = torch.from_numpy(m.init_k(KC0_SIZE)).to(dev)
    batch.quad4_update_KC0(Kr, Kc, Kv, x, cdof, ik, P, pid=pidt)
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    pat0 = CSRPattern(Kr, Kc, m.N, bk)
    torch.cuda.synchronize()
    t4 = time.perf_counter()
    v0 = pat0.assemble(Kv)
    same = bool((pat0.rowptr == pat.rowptr).all().item() and (pat0.colind == pat.colind).all().item())
    diff = float((vals - v0).abs().max().item() / v0.abs().max().item())

    def triplets():
        Kv.zero_()
        batch.quad4_update_KC0(Kr, Kc, Kv, x, cdof, ik, P, pid=pidt, check=False)
        pat0.assemble(Kv, out=v0)
    ms_t = timed(triplets, reps=3)
    ms_a = timed(lambda: pat0.assemble(Kv, out=v0), reps=3)
    out['triplet_path'] = {'ms_per_update': ms_t, 'assemble_ms': ms_a, 'pattern_from_triplets_s': t4 - t3,
                           'note': 'clearing of the COO values + update_KC0 (indices and values) + numeric '
                                   'assembly over the pattern'}
    out['same_pattern'] = same
    out['max_abs_diff_over_max_abs'] = diff
    out['speedup_vs_triplet_path'] = ms_t / out['assign']['ms_per_update']
    # bytes: inputs per element and the CSR values (written once at the least;
    # the coloured passes read and write every other contribution)
    in_bytes = 16 + 64 + 4 + 4 + 224 + 24
    out['bytes'] = {'csr_write_once_per_elem': pat.nnz * 8 / E + in_bytes,
                    'note': 'algorithmic minimum of the fused path: every CSR value written once plus the '
                            'element inputs (node ids, block offsets, assign bits, order, record, coordinates)'}
    peak = _peak_gbs()
    ach = (pat.nnz * 8 + E * in_bytes) / (out['assign']['ms_per_update'] / 1e3) / 1e9
    out['roofline_assign'] = {'achieved_gbs': ach, 'peak_gbs': peak, 'frac': ach / peak}
    # end to end with host buffers: the per-update inputs (coordinates, property
    # records, record ids) go host->device and the CSR values device->host (pinned
    # memory) in every timed update; pattern and map are built once beforehand
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    hx, hP, hpid = pin(m.x), pin(props), pin(pid)
    hvals = torch.empty(pat.nnz, dtype=torch.float64).pin_memory()
    dx, dP, dpid = torch.empty_like(x), torch.empty_like(P), torch.empty_like(pidt)

    def e2e_step():
        dx.copy_(hx, non_blocking=True)
        dP.copy_(hP, non_blocking=True)
        dpid.copy_(hpid, non_blocking=True)
        batch.quad4_update_KC0_csr(vals, fm, dx, dP, pid=dpid, check=False)
        hvals.copy_(vals, non_blocking=True)
    e2e_step()
    torch.cuda.synchronize()
    t5 = time.perf_counter()
    for _ in range(3):
        e2e_step()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t5) / 3
    assert torch.equal(hvals, vals.cpu())
    out['e2e_host_buffers'] = {'ms_per_update': dt * 1e3, 'elem_per_s': E / dt,
                               'h2d_bytes_per_step': int(hx.numel() * 8 + hP.numel() * 8 + hpid.numel() * 4),
                               'd2h_bytes_per_step': int(pat.nnz * 8),
                               'note': 'inputs up, fused KC0 into CSR, CSR values down, pinned buffers'}
    del hvals
    del Kr, Kc, Kv, v0, pat0
    torch.cuda.empty_cache()
    return out


def _peak_gbs():
    path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    try:
        with open(path) as fh:
            return float(json.load(fh)['hbm_gbs'])
    except Exception:  # noqa: BLE001 -- the recipe's fallback figure
        return 6800.0


def bench_solve(args):
    """Element -> CSR (fused) + block-Jacobi PCG to 1e-8 relative residual on
    the clamped perturbed plate generator at --solve-nodes: plain FP64,
    nested iterative refinement (inner FP32 PCG on the scaled system to 1e-2,
    outer FP64 residual), FP32 SpMV with FP64 reliable updates, and FP64 PCG
    with the split-FP32 SpMV (products on the FP32 pipe, float-float row
    sums, FP64 vectors and preconditioner); on the
    101x101-node plate also against scipy's spsolve on the host (the
    reference tests' solve)."""
    import torch
    from scipy.sparse.linalg import spsolve
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import config2
    from pyfe3d_gb300.solver import ElementPattern, FusedMap, Solver
    dev = torch.device('cuda')
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {}
    cases = [(101, True)] + ([(args.solve_nodes, False)] if args.solve_nodes != 101 else [])
    for n_nodes, small in cases:
        m, props, pid, bk, f = config2(n_nodes)
        cd = torch.from_numpy(m.cdof).to(dev)
        pat = ElementPattern([cd], m.N, bk)
        fm = FusedMap(pat, [cd])
        vals = batch.quad4_update_KC0_csr(fm.new_values(), fm, m.x, props, pid=pid)
        s = Solver(pat).setup(vals, mixed=True, split=True)
        fr = pat.reduce(f)
        res_case = {'workload': 'clamped perturbed plate %dx%d nodes' % (n_nodes, n_nodes),
                    'free_dofs': int(pat.nrows), 'nnz': int(pat.nnz)}
        uref = None
        if small and not args.no_cpu:
            A = pat.to_scipy(vals).tocsc()
            t0 = time.perf_counter()
            uref = spsolve(A, fr.cpu().numpy())
            res_case['cpu_spsolve_s'] = time.perf_counter() - t0
        u64 = None
        for name, prec, kw in (('plain_fp64', 0, {}),
                               ('nested_ir_fp32_inner', 3, {'inner_tol': 1e-2}),
                               ('fp32_spmv_reliable_updates', 1, {'replace_every': 400}),
                               ('split_fp32_spmv', 2, {})):
            if small:  # warm-up solve (graph capture) for the small case
                s.solve(fr, tol=1e-8, precision=prec, check_every=100, fallback=False, **kw)
            torch.cuda.synchronize()
            ev0.record()
            ur, st = s.solve(fr, tol=1e-8, precision=prec, check_every=100, maxiter=args.solve_maxiter, **kw)
            ev1.record()
            torch.cuda.synchronize()
            ms = ev0.elapsed_time(ev1)
            r = {'ms': ms, 'solves_per_s': 1e3 / ms, 'iterations': st['iterations'], 'relres': st['relres'],
                 'status': st['status'], 'outer_steps_or_replacements': st['replacements']}
            if 'fp64_iterations' in st:
                r['fp64_fallback_iterations'] = st['fp64_iterations']
            if uref is not None:
                r['relerr_vs_spsolve'] = float(np.linalg.norm(ur.cpu().numpy() - uref) / np.linalg.norm(uref))
            if prec == 0:
                u64 = ur
            elif u64 is not None:
                r['relerr_vs_fp64_pcg'] = float((ur - u64).norm().item() / u64.norm().item())
            res_case[name] = r
        b = res_case['plain_fp64']
        for name in ('nested_ir_fp32_inner', 'fp32_spmv_reliable_updates', 'split_fp32_spmv'):
            res_case[name]['iteration_ratio_vs_fp64'] = b['iterations'] / max(res_case[name]['iterations'], 1)
            res_case[name]['time_ratio_vs_fp64'] = b['ms'] / res_case[name]['ms']
        out['plate_%d' % n_nodes] = res_case
        del s, vals, fm, pat
        torch.cuda.empty_cache()
    return out


def bench_panel(args):
    """The stiffened panel at --panel-nel (default 500x500 elements: laminated
    Quad4 skin, 9 BeamC stringers of --panel-nel elements sharing its nodes,
    simply supported, in-plane compression plus lateral load): the pattern of
    both element groups from the connectivity, the skin's KC0 through the fused
    kernel and the stringers' values-only KC0 scattered by the same map, then
    block-Jacobi PCG to 1e-8 (plain FP64 and nested refinement); the 50x50
    panel is also solved with scipy's spsolve on the host for the error."""
    import torch
    from scipy.sparse.linalg import spsolve
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import config3
    from pyfe3d_gb300.solver import ElementPattern, FusedMap, Solver
    dev = torch.device('cuda')
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {}
    for nel, small in ((50, True), (args.panel_nel, False)):
        p = config3(nel)
        sk = p.skin
        groups = [torch.from_numpy(sk.cdof).to(dev), torch.from_numpy(p.beam_cdof).to(dev)]
        t0 = time.perf_counter()
        pat = ElementPattern(groups, p.N, p.bk)
        fm = FusedMap(pat, groups)
        torch.cuda.synchronize()
        setup_s = time.perf_counter() - t0
        x = torch.from_numpy(sk.x).to(dev)
        bik = torch.from_numpy(144 * np.arange(p.Eb, dtype=np.int64)).to(dev)
        kb = torch.zeros(144 * p.Eb, dtype=torch.float64, device=dev)
        vals = fm.new_values()

        def assemble():
            batch.quad4_update_KC0_csr(vals, fm, x, p.shell_props, group=0, check=False)
            kb.zero_()
            batch.beamc_update_KC0(None, None, kb, x, groups[1], bik, p.vxy, p.beam_props, update_KC0v_only=1,
                                   check=False)
            fm.scatter(vals, 1, bik, kb)
        assemble()
        torch.cuda.synchronize()
        ev0.record()
        assemble()
        ev1.record()
        torch.cuda.synchronize()
        res = {'workload': 'stiffened panel %dx%d Quad4 skin + 9 x %d BeamC stringers' % (nel, nel, nel),
               'quad4': int(p.Eq), 'beamc': int(p.Eb), 'free_dofs': int(pat.nrows), 'nnz': int(pat.nnz),
               'pattern_and_map_s': setup_s, 'assemble_ms': ev0.elapsed_time(ev1)}
        s = Solver(pat).setup(vals, mixed=True)
        fr = pat.reduce(p.f)
        uref = None
        if small and not args.no_cpu:
            t1 = time.perf_counter()
            uref = spsolve(pat.to_scipy(vals).tocsc(), fr.cpu().numpy())
            res['cpu_spsolve_s'] = time.perf_counter() - t1
        # nested refinement only on the small panel: on the full one it needs 14x the
        # iterations of FP64 (490,700 vs 35,400, 100 s; the laminate's kappa * eps32 is large)
        for name, prec in (('plain_fp64', 0),) + ((('nested_ir_fp32_inner', 3),) if small else ()):
            ev0.record()
            ur, st = s.solve(fr, tol=1e-8, precision=prec, check_every=100, maxiter=args.solve_maxiter)
            ev1.record()
            torch.cuda.synchronize()
            r = {'ms': ev0.elapsed_time(ev1), 'iterations': st['iterations'], 'relres': st['relres'],
                 'status': st['status']}
            if uref is not None:
                r['relerr_vs_spsolve'] = float(np.linalg.norm(ur.cpu().numpy() - uref) / np.linalg.norm(uref))
            res[name] = r
        out['panel_%d' % nel] = res
        del s, vals, fm, pat, kb
        torch.cuda.empty_cache()
    return out


def bench_batch(args):
    """Many independent uneven plates at the stated distribution (nx, ny
    uniform in [8, batch-nmax] elements): the block-diagonal pattern built
    from the elements, the fused KC0 of all plates into it, and the batched
    PCG.  The whole batch runs a capped number of lockstep iterations (rate
    per iteration); a seeded sample of plates is solved to 1e-8 batched and
    one plate at a time (plain FP64 PCG on the same GPU)."""
    import torch
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import BatchedPlates
    from pyfe3d_gb300.solver import BatchSolver, ElementPattern, FusedMap, Solver
    dev = torch.device('cuda')
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    bp = BatchedPlates(nplates=args.batch_plates, nmin=8, nmax=args.batch_nmax, seed=4)
    t1 = time.perf_counter()
    x, cdof = torch.from_numpy(bp.x).to(dev), torch.from_numpy(bp.cdof).to(dev)
    props, pid = torch.from_numpy(bp.props).to(dev), torch.from_numpy(bp.pid).to(dev)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    pat = ElementPattern([cdof], bp.N, bp.bk)
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    fm = FusedMap(pat, [cdof])
    torch.cuda.synchronize()
    t4 = time.perf_counter()
    vals = fm.new_values()
    batch.quad4_update_KC0_csr(vals, fm, x, props, pid=pid)
    torch.cuda.synchronize()
    ev0.record()
    batch.quad4_update_KC0_csr(vals, fm, x, props, pid=pid, check=False)
    ev1.record()
    torch.cuda.synchronize()
    kc0_ms = ev0.elapsed_time(ev1)
    out = {'workload': '%d isotropic plates, nx, ny uniform in [8, %d] elements, seeded' % (bp.P, args.batch_nmax),
           'elements': int(bp.E), 'free_dofs': int(pat.nrows), 'nnz': int(pat.nnz),
           'generate_s': t1 - t0, 'pattern_s': t3 - t2, 'map_s': t4 - t3,
           'kc0_into_csr_ms': kc0_ms, 'kc0_elem_per_s': bp.E / (kc0_ms / 1e3)}
    t5 = time.perf_counter()
    bs = BatchSolver(pat, bp.inst_of_dof, bp.P).setup(vals)
    torch.cuda.synchronize()
    out['solver_setup_s'] = time.perf_counter() - t5
    out['lanes_per_row'] = list(bs.lanes())
    fr = pat.reduce(bp.f)
    cap = args.batch_capped_iters
    ev0.record()
    ur, st = bs.solve(fr, tol=1e-8, precision=0, check_every=50, maxiter=cap)
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    out['all_plates_capped'] = {'maxiter': cap, 'ms': ms, 'ms_per_lockstep_iteration': ms / max(st['iterations'], 1),
                                'converged': int((st['inst_status'] == 0).sum()),
                                'note': 'every plate of the batch for a capped number of lockstep FP64 iterations'}
    del bs, ur, vals, fm, pat
    torch.cuda.empty_cache()
    # seeded sample of the same plates: batched and one at a time, to 1e-8
    rng = np.random.default_rng(5)
    sample = np.sort(rng.choice(bp.P, size=min(args.batch_sample, bp.P), replace=False))
    sub = bp.subset(sample)
    scd = torch.from_numpy(sub.cdof).to(dev)
    spat = ElementPattern([scd], sub.N, sub.bk)
    sfm = FusedMap(spat, [scd])
    svals = batch.quad4_update_KC0_csr(sfm.new_values(), sfm, sub.x, sub.props, pid=sub.pid)
    sbs = BatchSolver(spat, sub.inst_of_dof, sub.P).setup(svals)
    sfr = spat.reduce(sub.f)
    sbs.solve(sfr, tol=1e-8, precision=0, check_every=50, maxiter=100)
    torch.cuda.synchronize()
    ev0.record()
    ur, st = sbs.solve(sfr, tol=1e-8, precision=0, check_every=50)
    ev1.record()
    torch.cuda.synchronize()
    ms_b = ev0.elapsed_time(ev1)
    res = {'sample_plates': int(sub.P), 'sample_elements': int(sub.E),
           'batched_fp64': {'ms': ms_b, 'solves_per_s': sub.P * 1e3 / ms_b, 'lockstep_iterations': st['iterations'],
                            'max_plate_iterations': int(st['inst_iters'].max()),
                            'mean_plate_iterations': float(st['inst_iters'].mean()),
                            'max_relres': float(st['inst_relres'].max()),
                            'converged': int((st['inst_status'] == 0).sum())}}
    total_ms, iters = 0., []
    for i in range(sub.P):
        pc = sub.plate(i)
        pcd = torch.from_numpy(pc.cdof).to(dev)
        p1 = ElementPattern([pcd], pc.N, pc.bk)
        f1m = FusedMap(p1, [pcd])
        v1 = batch.quad4_update_KC0_csr(f1m.new_values(), f1m, pc.x, pc.props, pid=pc.pid)
        s1 = Solver(p1).setup(v1)
        f1 = p1.reduce(pc.f)
        s1.solve(f1, tol=1e-8, check_every=50, maxiter=100)
        torch.cuda.synchronize()
        ev0.record()
        _, st1 = s1.solve(f1, tol=1e-8, check_every=50)
        ev1.record()
        torch.cuda.synchronize()
        total_ms += ev0.elapsed_time(ev1)
        iters.append(st1['iterations'])
    res['one_at_a_time_fp64'] = {'ms': total_ms, 'solves_per_s': sub.P * 1e3 / total_ms,
                                 'mean_iterations': float(np.mean(iters)), 'max_iterations': int(np.max(iters))}
    res['batched_speedup'] = total_ms / ms_b
    out['sample_to_1e-8'] = res
    out['work_split'] = bench_work_split()
    return out


def bench_work_split():
    """The batched solver's work split on many small plates: every plate in
    the lockstep recurrence, against every plate solved by one thread block
    of the block-resident kernel, to 1e-8 in FP64; with the SpMV FMAs each
    run performed (sum over plates of iterations x nonzeros) and their rate."""
    import torch
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import BatchedPlates
    from pyfe3d_gb300.solver import BatchSolver, ElementPattern, FusedMap
    dev = torch.device('cuda')
    bp = BatchedPlates(nplates=1024, nmin=4, nmax=12, seed=6)
    cd = torch.from_numpy(bp.cdof).to(dev)
    pat = ElementPattern([cd], bp.N, bp.bk)
    fm = FusedMap(pat, [cd])
    vals = batch.quad4_update_KC0_csr(fm.new_values(), fm, bp.x, bp.props, pid=bp.pid)
    bs = BatchSolver(pat, bp.inst_of_dof, bp.P).setup(vals)
    fr = pat.reduce(bp.f)
    inst = bs.inst_of_row.long()
    rows = torch.bincount(inst, minlength=bp.P).cpu().numpy()
    row_nnz = (pat.rowptr[1:] - pat.rowptr[:-1]).double()
    nnz = torch.bincount(inst, weights=row_nnz, minlength=bp.P).cpu().numpy()
    out = {'workload': '%d isotropic plates, nx, ny uniform in [4, 12] elements, seeded' % bp.P,
           'free_dofs': int(pat.nrows), 'nnz': int(pat.nnz), 'max_plate_rows': int(rows.max())}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for name, split in (('lockstep', 0), ('block_resident', int(rows.max()))):
        bs.set_split(split)
        bs.solve(fr, tol=1e-8, check_every=50, maxiter=50)
        torch.cuda.synchronize()
        ev0.record()
        _, st = bs.solve(fr, tol=1e-8, check_every=50)
        ev1.record()
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        fma = float((st['inst_iters'] * nnz).sum())
        out[name] = {'ms': ms, 'solves_per_s': bp.P * 1e3 / ms, 'converged': int((st['inst_status'] == 0).sum()),
                     'max_relres': float(st['inst_relres'].max()), 'max_plate_iterations': int(st['inst_iters'].max()),
                     'spmv_fp64_fma': fma, 'spmv_fp64_tflops': 2 * fma / (ms / 1e3) / 1e12}
    out['note'] = ('both paths are bound by the slowest plates: their iterations times the latency of one '
                   'iteration (lockstep: three graph-launched kernels; block-resident: dependent row trips '
                   'inside one block), not by FP64 throughput or bandwidth (see spmv_fp64_tflops)')
    return out


def bench_learned(args):
    """Learned block preconditioner: residual/error pairs from the FP64 solver
    on seeded random-thickness plates, training with the library's CUDA
    kernels for both input sets (35 features; the 29 of the normalised
    diagonal block and neighbour-block norms), then on a held-out plate plain
    block-Jacobi PCG against PCG with the learned blocks (flexible and plain),
    all to 1e-8 relative residual in FP64, and the block-diagonal ceiling:
    free per-node blocks fitted on the held-out plate itself."""
    import torch
    from pyfe3d_gb300 import batch, learned
    from pyfe3d_gb300.meshes import RandomFieldPlate
    from pyfe3d_gb300.solver import ElementPattern, FusedMap, Solver
    dev = torch.device('cuda')

    def system(p):
        cd = torch.from_numpy(p.cdof).to(dev)
        pat = ElementPattern([cd], p.N, p.bk)
        fm = FusedMap(pat, [cd])
        return pat, batch.quad4_update_KC0_csr(fm.new_values(), fm, p.x, p.props, pid=p.pid)

    rng = np.random.default_rng(6)
    t0 = time.perf_counter()
    systems = []
    for k in range(args.lpc_train_plates):
        p = RandomFieldPlate(int(rng.integers(args.lpc_train_min, args.lpc_train_max + 1)), seed=1000 + k)
        pat, vals = system(p)
        systems.append(learned.make_training_system(pat, vals, pat.reduce(p.f), npairs=args.lpc_pairs))
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    pcs = {}
    out = {'pairs': int(sum(len(s.samples) for s in systems)), 'pair_generation_s': t1 - t0,
           'steps': args.lpc_steps}
    for fs in (0, 1):
        ta = time.perf_counter()
        pc = learned.LearnedPC(seed=0, out_scale=0.1, feature_set=fs)
        before = pc.evaluate(systems)
        pc.train(systems, steps=args.lpc_steps, batch=8, lr=2e-3)
        after = pc.evaluate(systems)
        torch.cuda.synchronize()
        pcs[fs] = pc
        out['training_features_%d' % (35 if fs == 0 else 29)] = {
            'objective_block_jacobi': before, 'objective_trained': after, 'training_s': time.perf_counter() - ta}
    p = RandomFieldPlate(args.lpc_nel, seed=424242)
    pat, vals = system(p)
    fr = pat.reduce(p.f)
    out['workload'] = ('held-out random-thickness plate %dx%d elements; training on %d plates of %d..%d elements a side'
                       % (args.lpc_nel, args.lpc_nel, args.lpc_train_plates, args.lpc_train_min, args.lpc_train_max))
    out['free_dofs'] = int(pat.nrows)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def run(name, setup, flex):
        s = Solver(pat).setup(vals)
        nfb = setup(s)
        s.solve(fr, tol=1e-8, check_every=100, flexible=flex, maxiter=200)
        torch.cuda.synchronize()
        ev0.record()
        ur, st = s.solve(fr, tol=1e-8, check_every=100, flexible=flex)
        ev1.record()
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        out[name] = {'ms': ms, 'solves_per_s': 1e3 / ms, 'iterations': st['iterations'], 'relres': st['relres'],
                     'status': st['status'], 'fallback_nodes': int(nfb)}

    run('block_jacobi_fp64', lambda s: 0, False)
    for fs, tag in ((0, '35'), (1, '29')):
        run('learned%s_flexible_fp64' % tag, lambda s, fs=fs: pcs[fs].install(s), True)
        run('learned%s_plain_fp64' % tag, lambda s, fs=fs: pcs[fs].install(s), False)
    b = out['block_jacobi_fp64']
    for k in list(out):
        if isinstance(out[k], dict) and 'iterations' in out[k] and k != 'block_jacobi_fp64':
            out[k]['iteration_ratio_vs_block_jacobi'] = b['iterations'] / max(out[k]['iterations'], 1)
            out[k]['time_ratio_vs_block_jacobi'] = b['ms'] / out[k]['ms']
    # the ceiling of any block-diagonal preconditioner on a small plate
    if args.lpc_bound_nel > 0:
        out['block_diagonal_ceiling'] = kappa_bound(args, pcs[0], system)
    return out


def _node_rows(dof_of_row, nnodes):
    rows = [[] for _ in range(nnodes)]
    for r, d in enumerate(dof_of_row):
        rows[int(d) // 6].append(r)
    return [np.array(r, dtype=np.int64) for r in rows]


def _pencil_kappa(K, B):
    from scipy.linalg import eigh
    w = eigh(K, B, eigvals_only=True)
    return w[-1] / w[0]


def kappa_bound(args, pc, system):
    """Block-diagonal ceiling on a small random-thickness plate: the
    condition number of B^-1 K for block Jacobi, for the learned blocks and
    for block-diagonal SPD B minimised directly (host, dense generalised
    eigenproblems: Riemannian gradient steps on a smoothed log(lmax/lmin)
    with backtracking, from block Jacobi), then PCG iterations to 1e-8 on
    the GPU with each.  No block-diagonal preconditioner does better than
    the minimised one on this plate (up to the optimiser's convergence)."""
    import torch
    from scipy.linalg import eigh
    from pyfe3d_gb300 import learned
    from pyfe3d_gb300.meshes import RandomFieldPlate
    from pyfe3d_gb300.solver import Solver
    t0 = time.perf_counter()
    p = RandomFieldPlate(args.lpc_bound_nel, seed=77)
    pat, vals = system(p)
    K = pat.to_scipy(vals).toarray()
    n = K.shape[0]
    nn = (pat.N + 5) // 6
    rows = _node_rows(pat.dof_of_row.cpu().numpy(), nn)

    def dense(blocks):
        B = np.zeros((n, n))
        for j, r in enumerate(rows):
            if len(r):
                B[np.ix_(r, r)] = blocks[j]
        return B

    bj = [K[np.ix_(r, r)] if len(r) else np.zeros((0, 0)) for r in rows]

    def objective(blocks, t=40.):
        w, V = eigh(K, dense(blocks))
        lw = np.log(w)
        pmax = np.exp(t * (lw - lw.max()))
        pmax /= pmax.sum()
        pmin = np.exp(-t * (lw - lw.min()))
        pmin /= pmin.sum()
        f = lw.max() + np.log(np.exp(t * (lw - lw.max())).sum()) / t - \
            (lw.min() - np.log(np.exp(-t * (lw - lw.min())).sum()) / t)
        return f, w, V, pmax - pmin

    blocks = [b.copy() for b in bj]
    f, w, V, c = objective(blocks)
    kappa_bj = w[-1] / w[0]
    eta = 0.5
    for it in range(args.lpc_bound_steps):
        G = [-(V[r] * c) @ V[r].T if len(r) else None for r in rows]
        while eta > 1e-8:
            trial = []
            ok = True
            for b, g in zip(blocks, G):
                if g is None:
                    trial.append(b)
                    continue
                nb = b - eta * b @ g @ b
                nb = 0.5 * (nb + nb.T)
                if np.linalg.eigvalsh(nb).min() <= 0:
                    ok = False
                    break
                trial.append(nb)
            if ok:
                f2, w2, V2, c2 = objective(trial)
                if f2 < f:
                    blocks, f, w, V, c = trial, f2, w2, V2, c2
                    eta *= 1.5
                    break
            eta *= 0.5
        if eta <= 1e-8:
            break
    kappa_opt = w[-1] / w[0]
    # the learned network's blocks on this plate
    s_l = Solver(pat).setup(vals)
    ctx = learned._Ctx(s_l, pc.feature_set)
    pc._forward_blocks(ctx, train=False)
    lb = ctx.blocks.cpu().numpy().reshape(nn, 6, 6)
    kappa_learned = _pencil_kappa(K, dense([lb[j][:len(r), :len(r)] for j, r in enumerate(rows)]))
    dev = torch.device('cuda')
    fr = pat.reduce(p.f)

    def iters(blocks_list):
        s = Solver(pat).setup(vals)
        if blocks_list is not None:
            arr = np.zeros((nn, 6, 6))
            for j, (r, b) in enumerate(zip(rows, blocks_list)):
                arr[j, :len(r), :len(r)] = b
            learned.install_blocks(s, torch.from_numpy(arr.ravel()).to(dev))
        _, st = s.solve(fr, tol=1e-8, check_every=2)
        return st['iterations']

    it_bj, it_opt = iters(None), iters(blocks)
    _, st_l = s_l.solve(fr, tol=1e-8, check_every=2)
    return {'workload': 'random-thickness plate %dx%d elements (%d free DOFs)' % (args.lpc_bound_nel,
                                                                                args.lpc_bound_nel, n),
            'kappa_block_jacobi': float(kappa_bj), 'kappa_learned': float(kappa_learned),
            'kappa_minimised_block_diagonal': float(kappa_opt),
            'kappa_ratio_best_found': float(kappa_bj / kappa_opt),
            'cg_bound_iteration_ratio': float(np.sqrt(kappa_bj / kappa_opt)),
            'iterations_block_jacobi': int(it_bj), 'iterations_learned': int(st_l['iterations']),
            'iterations_minimised_block_diagonal': int(it_opt),
            'note': ('kappa of the preconditioned operator; the CG bound on the iteration ratio is the square '
                     'root of the kappa ratio; iteration counts to 1e-8 also depend on the rest of the spectrum'),
            'seconds': time.perf_counter() - t0}


def run_e2e(args, m, props, pid):
    """update_KC0 through pyfe3d_gb300.batch with pinned host buffers: the
    inputs (coordinates, offsets, properties, current values) go host->device
    and the triplets device->host inside every timed step."""
    import torch
    from pyfe3d_gb300 import batch
    E = m.E
    n = KC0_SIZE * E
    pin = lambda a: torch.from_numpy(a).pin_memory()
    x, cdof, ik = pin(m.x), pin(m.cdof), pin(m.init_k(KC0_SIZE))
    P, pidt = pin(props), pin(pid)
    Kr = torch.zeros(n, dtype=torch.int64).pin_memory()
    Kc = torch.zeros(n, dtype=torch.int64).pin_memory()
    Kv = torch.zeros(n, dtype=torch.float64).pin_memory()
    for _ in range(2):
        batch.quad4_update_KC0(Kr, Kc, Kv, x, cdof, ik, P, pid=pidt)
    torch.cuda.synchronize()
    steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(steps):
        batch.quad4_update_KC0(Kr, Kc, Kv, x, cdof, ik, P, pid=pidt)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    # bytes the pipelined host path moves per step (init_k is only checked on
    # the host for the contiguous layout; every slot is written)
    h2d = sum(t.numel() * t.element_size() for t in (x, cdof, P, pidt, Kv))
    d2h = sum(t.numel() * t.element_size() for t in (Kr, Kc, Kv))
    # values only (update_KC0v_only=1, the reference's optimisation-loop use):
    # the indices stay as they are and only the values move down
    batch.quad4_update_KC0(Kr, Kc, Kv, x, cdof, ik, P, pid=pidt, update_KC0v_only=1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        batch.quad4_update_KC0(Kr, Kc, Kv, x, cdof, ik, P, pid=pidt, update_KC0v_only=1)
    torch.cuda.synchronize()
    dtv = (time.perf_counter() - t0) / steps
    values_only = {'value': E / dtv, 'unit': 'elem/s', 'ms_per_step': dtv * 1e3,
                   'h2d_bytes_per_step': sum(t.numel() * t.element_size() for t in (x, cdof, P, pidt, Kv)),
                   'd2h_bytes_per_step': Kv.numel() * Kv.element_size()}
    # the host link's device->host copy rate (copy engines, pinned memory):
    # the bound of this step, which moves more bytes down than up
    # (best of five 1 GiB copies into the step's own pinned value buffer)
    dv = torch.empty(1 << 27, dtype=torch.float64, device='cuda')
    hv = Kv[:1 << 27]
    hv.copy_(dv, non_blocking=True)
    torch.cuda.synchronize()
    link = 0.
    for _ in range(5):
        t1 = time.perf_counter()
        hv.copy_(dv, non_blocking=True)
        torch.cuda.synchronize()
        link = max(link, dv.numel() * 8 / (time.perf_counter() - t1) / 1e9)
    del dv
    return {'value': E / dt, 'unit': 'elem/s', 'h2d_bytes_per_step': h2d,
            'd2h_bytes_per_step': d2h, 'ms_per_step': dt * 1e3,
            'link_d2h_gbs': link, 'link_bound_ms': d2h / link / 1e6, 'values_only': values_only}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--nodes', type=int, default=1001)
    ap.add_argument('--ref-seconds', type=float, default=12.0)
    ap.add_argument('--ref-workers', type=int, default=0,
                    help='processes of the reference arm (default: every host core)')
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--traffic-per-launch', type=float, default=None,
                    help='DRAM bytes per launch from an ncu capture (default: the committed '
                         'profile scaled to the element count)')
    ap.add_argument('--no-fused', action='store_true')
    ap.add_argument('--solve-nodes', type=int, default=501)
    ap.add_argument('--no-solve', action='store_true')
    ap.add_argument('--no-other', action='store_true')
    ap.add_argument('--solve-maxiter', type=int, default=1000000)
    ap.add_argument('--no-batch', action='store_true')
    ap.add_argument('--no-panel', action='store_true')
    ap.add_argument('--panel-nel', type=int, default=500)
    ap.add_argument('--batch-plates', type=int, default=1024)
    ap.add_argument('--batch-nmax', type=int, default=256)
    ap.add_argument('--batch-sample', type=int, default=24)
    ap.add_argument('--batch-capped-iters', type=int, default=100)
    ap.add_argument('--no-learned', action='store_true')
    ap.add_argument('--lpc-train-plates', type=int, default=8)
    ap.add_argument('--lpc-train-min', type=int, default=32)
    ap.add_argument('--lpc-train-max', type=int, default=64)
    ap.add_argument('--lpc-pairs', type=int, default=32)
    ap.add_argument('--lpc-steps', type=int, default=1500)
    ap.add_argument('--lpc-nel', type=int, default=100)
    ap.add_argument('--lpc-bound-steps', type=int, default=300)
    ap.add_argument('--lpc-bound-nel', type=int, default=8)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()
    if args.impl == 'reference':
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == '__main__':
    main()
