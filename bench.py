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
# DRAM bytes per element measured by ncu on a 90,000-element launch
# (444.2 MB read + 1188.5 MB written)
TRAFFIC_PER_ELEM = (444.509696e6 + 1197.154e6) / 90000


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


def cpu_baseline(m, props, pid, seconds=12.0, threads=None):
    """Time the CPU oracle on a bounded prefix of the same elements."""
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
    if rank != 0:
        return
    m, props, pid = workload(args.nodes)
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
        out['cpu_baseline'] = cpu_baseline(m, props, pid, seconds=args.ref_seconds)
    # the sections after the headline measurement report their own failure
    # instead of losing the line
    for key, skip, fn in (('other_kernels', args.no_other, bench_other_kernels),
                          ('solve', args.no_solve, bench_solve),
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


def bench_solve(args):
    """Assembly + BC elimination + block-Jacobi PCG to 1e-8 relative residual
    on the clamped perturbed plate generator at --solve-nodes, FP64 and
    mixed precision, against scipy's spsolve (the reference tests' solve) on
    the same reduced matrix."""
    import torch
    from scipy.sparse.linalg import spsolve
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import config2
    from pyfe3d_gb300.solver import CSRPattern, Solver
    n_nodes = args.solve_nodes
    m, props, pid, bk, f = config2(n_nodes)
    dev = torch.device('cuda')
    nk = KC0_SIZE * m.E
    Kr = torch.zeros(nk, dtype=torch.int64, device=dev)
    Kc = torch.zeros(nk, dtype=torch.int64, device=dev)
    Kv = torch.zeros(nk, dtype=torch.float64, device=dev)
    batch.quad4_update_KC0(Kr, Kc, Kv, m.x, m.cdof, m.init_k(KC0_SIZE), props, pid=pid)
    pat = CSRPattern(Kr, Kc, m.N, bk)
    vals = pat.assemble(Kv)
    torch.cuda.synchronize()
    # numeric re-assembly time (pattern reused)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(5):
        pat.assemble(Kv, out=vals)
    ev1.record()
    torch.cuda.synchronize()
    assemble_ms = ev0.elapsed_time(ev1) / 5
    s = Solver(pat).setup(vals, mixed=True, split=True)
    fr = pat.reduce(f)
    out = {'workload': 'clamped perturbed plate %dx%d nodes' % (n_nodes, n_nodes),
           'free_dofs': int(pat.nrows), 'nnz': int(pat.nnz), 'assemble_ms': assemble_ms}
    A = None
    uref = None
    if not args.no_cpu and pat.nrows <= 300000:
        A = pat.to_scipy(vals).tocsc()
        frh = fr.cpu().numpy()
        t0 = time.perf_counter()
        uref = spsolve(A, frh)
        out['cpu_spsolve_s'] = time.perf_counter() - t0
    for name, prec in (('plain_fp64', 0), ('mixed_fp32_spmv', 1), ('fp64_split_spmv', 2)):
        if pat.nrows < 1000000:  # warm-up solve (graph capture) for the small case
            ur, st = s.solve(fr, tol=1e-8, precision=prec, check_every=100, replace_every=400)
        torch.cuda.synchronize()
        ev0.record()
        ur, st = s.solve(fr, tol=1e-8, precision=prec, check_every=100, replace_every=400,
                         maxiter=args.solve_maxiter)
        ev1.record()
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        res = {'ms': ms, 'solves_per_s': 1e3 / ms, 'iterations': st['iterations'],
               'relres': st['relres'], 'status': st['status'], 'replacements': st['replacements']}
        if uref is not None:
            res['relerr_vs_spsolve'] = float(np.linalg.norm(ur.cpu().numpy() - uref) / np.linalg.norm(uref))
        out[name] = res
    return out


def bench_batch(args):
    """Many independent uneven plates: KC0 of all plates in one launch,
    one pattern of the block-diagonal system, and the batched PCG to 1e-8
    on every plate (FP32 SpMV with FP64 residual replacement, and plain FP64),
    against one-at-a-time plain FP64 PCG on the same GPU timed on a seeded
    sample of plates and extrapolated to all of them."""
    import torch
    from pyfe3d_gb300 import batch
    from pyfe3d_gb300.meshes import BatchedPlates
    from pyfe3d_gb300.solver import BatchSolver, CSRPattern, Solver
    bp = BatchedPlates(nplates=args.batch_plates, nmin=8, nmax=args.batch_nmax, seed=4)
    dev = torch.device('cuda')
    nk = KC0_SIZE * bp.E
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    Kr = torch.zeros(nk, dtype=torch.int64, device=dev)
    Kc = torch.zeros(nk, dtype=torch.int64, device=dev)
    Kv = torch.zeros(nk, dtype=torch.float64, device=dev)
    x, cdof, ik = (torch.from_numpy(a).to(dev) for a in (bp.x, bp.cdof, bp.init_k(KC0_SIZE)))
    props, pid = torch.from_numpy(bp.props).to(dev), torch.from_numpy(bp.pid).to(dev)
    batch.quad4_update_KC0(Kr, Kc, Kv, x, cdof, ik, props, pid=pid)
    pat = CSRPattern(Kr, Kc, bp.N, bp.bk)
    vals = pat.assemble(Kv)
    torch.cuda.synchronize()
    ev0.record()
    Kv.zero_()
    batch.quad4_update_KC0(Kr, Kc, Kv, x, cdof, ik, props, pid=pid)
    pat.assemble(Kv, out=vals)
    ev1.record()
    torch.cuda.synchronize()
    kc0_assemble_ms = ev0.elapsed_time(ev1)
    bs = BatchSolver(pat, bp.inst_of_dof, bp.P).setup(vals, mixed=True)
    fr = pat.reduce(bp.f)
    out = {'workload': '%d isotropic plates, nx, ny uniform in [8, %d] nodes, seeded' % (bp.P, args.batch_nmax),
           'elements': int(bp.E), 'free_dofs': int(pat.nrows), 'nnz': int(pat.nnz),
           'kc0_plus_assemble_ms': kc0_assemble_ms, 'lanes_per_row': list(bs.lanes())}
    for name, prec in (('batched_mixed', 1), ('batched_fp64', 0)):
        bs.solve(fr, tol=1e-8, precision=prec, check_every=50, replace_every=200, maxiter=100)
        torch.cuda.synchronize()
        ev0.record()
        ur, st = bs.solve(fr, tol=1e-8, precision=prec, check_every=50, replace_every=200)
        ev1.record()
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        out[name] = {'ms': ms, 'solves_per_s': bp.P * 1e3 / ms, 'lockstep_iterations': st['iterations'],
                     'max_plate_iterations': int(st['inst_iters'].max()),
                     'mean_plate_iterations': float(st['inst_iters'].mean()),
                     'max_relres': float(st['inst_relres'].max()),
                     'converged': int((st['inst_status'] == 0).sum()), 'replacements': st['replacements'],
                     'fp64_fallback_plates': int(st.get('fp64_instances', 0))}
    # one at a time: plain FP64 PCG per plate (pattern and setup outside the
    # timed region, as for the batch)
    rng = np.random.default_rng(5)
    sample = np.sort(rng.choice(bp.P, size=min(args.batch_sample, bp.P), replace=False))
    total_ms, iters = 0., []
    for i in sample:
        e = slice(int(bp.elem0[i]), int(bp.elem0[i + 1]))
        d = bp.plate_dofs(i)
        lo, hi = KC0_SIZE * e.start, KC0_SIZE * e.stop
        r1 = Kr[lo:hi] - int(bp.dof0[i])
        c1 = Kc[lo:hi] - int(bp.dof0[i])
        p1 = CSRPattern(r1, c1, d.stop - d.start, bp.bk[d])
        s1 = Solver(p1).setup(p1.assemble(Kv[lo:hi]))
        f1 = p1.reduce(bp.f[d])
        s1.solve(f1, tol=1e-8, check_every=50, maxiter=100)
        torch.cuda.synchronize()
        ev0.record()
        _, st1 = s1.solve(f1, tol=1e-8, check_every=50)
        ev1.record()
        torch.cuda.synchronize()
        total_ms += ev0.elapsed_time(ev1)
        iters.append(st1['iterations'])
    out['one_at_a_time_fp64'] = {'sample_plates': int(sample.size), 'sample_ms': total_ms,
                                 'solves_per_s': sample.size * 1e3 / total_ms,
                                 'mean_iterations': float(np.mean(iters)),
                                 'note': 'extrapolated from the sample to all plates'}
    return out


def bench_learned(args):
    """Learned block preconditioner: pairs from the FP64 solver on seeded
    random-thickness plates, training with the library's CUDA kernels, then
    on a held-out plate plain block-Jacobi PCG against flexible PCG with the
    learned blocks, both to 1e-8 relative residual (FP64 and mixed)."""
    import torch
    from pyfe3d_gb300 import batch, learned
    from pyfe3d_gb300.meshes import RandomFieldPlate
    from pyfe3d_gb300.solver import CSRPattern, Solver
    dev = torch.device('cuda')

    def system(p):
        nk = KC0_SIZE * p.E
        Kr = torch.zeros(nk, dtype=torch.int64, device=dev)
        Kc = torch.zeros(nk, dtype=torch.int64, device=dev)
        Kv = torch.zeros(nk, dtype=torch.float64, device=dev)
        batch.quad4_update_KC0(Kr, Kc, Kv, p.x, p.cdof, p.init_k(KC0_SIZE), p.props, pid=p.pid)
        pat = CSRPattern(Kr, Kc, p.N, p.bk)
        return pat, pat.assemble(Kv)

    rng = np.random.default_rng(6)
    t0 = time.perf_counter()
    systems = []
    for k in range(args.lpc_train_plates):
        p = RandomFieldPlate(int(rng.integers(args.lpc_train_min, args.lpc_train_max + 1)), seed=1000 + k)
        pat, vals = system(p)
        systems.append(learned.make_training_system(pat, vals, pat.reduce(p.f), npairs=args.lpc_pairs))
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    pc = learned.LearnedPC(seed=0, out_scale=0.1)
    before = pc.evaluate(systems)
    pc.train(systems, steps=args.lpc_steps, batch=8, lr=2e-3)
    after = pc.evaluate(systems)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    p = RandomFieldPlate(args.lpc_nel, seed=424242)
    pat, vals = system(p)
    fr = pat.reduce(p.f)
    out = {'workload': 'held-out random-thickness plate %dx%d elements; training on %d plates of %d..%d'
                       % (args.lpc_nel, args.lpc_nel, args.lpc_train_plates, args.lpc_train_min, args.lpc_train_max),
           'free_dofs': int(pat.nrows), 'pairs': int(sum(len(s.samples) for s in systems)),
           'pair_generation_s': t1 - t0, 'training_s': t2 - t1, 'steps': args.lpc_steps,
           'objective_block_jacobi': before, 'objective_trained': after}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    precs = [int(v) for v in args.lpc_precisions.split(',')]
    # learned blocks in flexible CG (the safe form for any preconditioner) and
    # in plain PCG (valid too: the installed blocks are symmetric positive
    # definite, per node by Cholesky, else block Jacobi)
    for name, learned_on, flex, prec in (('block_jacobi_fp64', False, False, 0),
                                         ('learned_flexible_fp64', True, True, 0),
                                         ('learned_plain_fp64', True, False, 0),
                                         ('block_jacobi_mixed', False, False, 1),
                                         ('learned_flexible_mixed', True, True, 1)):
        if prec not in precs:
            continue
        s = Solver(pat).setup(vals, mixed=(prec == 1))
        nfb = pc.install(s) if learned_on else 0
        s.solve(fr, tol=1e-8, precision=prec, check_every=100, replace_every=400, flexible=flex, maxiter=200)
        torch.cuda.synchronize()
        ev0.record()
        ur, st = s.solve(fr, tol=1e-8, precision=prec, check_every=100, replace_every=400, flexible=flex)
        ev1.record()
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        out[name] = {'ms': ms, 'solves_per_s': 1e3 / ms, 'iterations': st['iterations'], 'relres': st['relres'],
                     'status': st['status'], 'fallback_nodes': int(nfb)}
    if 'block_jacobi_fp64' in out and 'learned_flexible_fp64' in out:
        b, l = out['block_jacobi_fp64']['iterations'], out['learned_flexible_fp64']['iterations']
        out['iteration_ratio_fp64'] = b / l if l else None
        out['time_ratio_fp64'] = out['block_jacobi_fp64']['ms'] / out['learned_flexible_fp64']['ms']
    if 'block_jacobi_fp64' in out and 'learned_plain_fp64' in out:
        out['time_ratio_plain_fp64'] = out['block_jacobi_fp64']['ms'] / out['learned_plain_fp64']['ms']
    return out


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
            'link_d2h_gbs': link, 'link_bound_ms': d2h / link / 1e6}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--nodes', type=int, default=1001)
    ap.add_argument('--ref-seconds', type=float, default=12.0)
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--traffic-per-launch', type=float, default=None,
                    help='DRAM bytes per launch from an ncu capture (default: the committed '
                         'profile scaled to the element count)')
    ap.add_argument('--solve-nodes', type=int, default=101)
    ap.add_argument('--no-solve', action='store_true')
    ap.add_argument('--no-other', action='store_true')
    ap.add_argument('--solve-maxiter', type=int, default=1000000)
    ap.add_argument('--no-batch', action='store_true')
    ap.add_argument('--batch-plates', type=int, default=1024)
    ap.add_argument('--batch-nmax', type=int, default=32)
    ap.add_argument('--batch-sample', type=int, default=16)
    ap.add_argument('--no-learned', action='store_true')
    ap.add_argument('--lpc-train-plates', type=int, default=8)
    ap.add_argument('--lpc-train-min', type=int, default=32)
    ap.add_argument('--lpc-train-max', type=int, default=64)
    ap.add_argument('--lpc-pairs', type=int, default=32)
    ap.add_argument('--lpc-steps', type=int, default=1500)
    ap.add_argument('--lpc-nel', type=int, default=100)
    ap.add_argument('--lpc-precisions', default='0,1')
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()
    if args.impl == 'reference':
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == '__main__':
    main()
