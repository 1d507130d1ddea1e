"""Learned block preconditioner: a per-node MLP that corrects each 6x6
block-Jacobi block, trained and evaluated on the GPU with the library's own
CUDA kernels (fe3d_lpc_*), used inside flexible CG.

No counterpart in the reference, whose tests solve with spsolve/cg
(tests/test_quad4_static_point_load.py:102).  A poor network costs
iterations only: the solve still stops on the FP64 residual, and blocks
that are not positive definite fall back to block Jacobi.

Typical use::

    pc = LearnedPC()
    data = [make_training_system(pattern, vals, f) for ...]   # FP64 solver pairs
    pc.train(data, steps=2000)
    solver = Solver(pattern).setup(vals)
    pc.install(solver)
    u, stats = solver.solve(f, flexible=True)
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import c_int

NF, NH, NO, NW = 35, 64, 21, 7829


def init_weights(seed=0, out_std=0.0):
    """Random hidden layers; output layer scaled by out_std (0: the network
    starts as plain block Jacobi)."""
    rng = np.random.default_rng(seed)
    W = np.zeros(NW, dtype=np.float32)
    W[0:NH * NF] = rng.normal(0, 1 / np.sqrt(NF), NH * NF)
    o2 = NH * NF + NH
    W[o2:o2 + NH * NH] = rng.normal(0, 1 / np.sqrt(NH), NH * NH)
    o3 = o2 + NH * NH + NH
    W[o3:o3 + NO * NH] = rng.normal(0, out_std / np.sqrt(NH), NO * NH) if out_std > 0 else 0.
    return W


class _Ctx:
    """Device buffers of one system (solver) for the learned preconditioner."""

    def __init__(self, solver, feature_set=0):
        torch = _lib.torch_mod()
        lib = _lib.load()
        dev = _lib.device()
        s = solver
        self.solver = s
        self.n = s.pattern.nrows
        self.nnodes = (s.pattern.N + 5) // 6
        nn = self.nnodes
        self.feat = torch.zeros(max(nn, 1) * NF, dtype=torch.float32, device=dev)
        self.sdiag = torch.ones(max(self.n, 1), dtype=torch.float64, device=dev)
        self.out = torch.zeros(max(nn, 1) * NO, dtype=torch.float32, device=dev)
        self.act = None
        self.blocks = torch.zeros(max(nn, 1) * 36, dtype=torch.float64, device=dev)
        self.fallback = torch.zeros(max(nn, 1), dtype=torch.int8, device=dev)
        self.feature_set = int(feature_set)
        rc = lib.fe3d_lpc_features_set(s._h, self.feature_set, _lib.ptr(self.feat), _lib.ptr(self.sdiag),
                                       _lib.stream_ptr())
        _lib.check(rc, 'fe3d_lpc_features_set')

    def train_buffers(self):
        torch = _lib.torch_mod()
        dev = _lib.device()
        if self.act is None:
            nn = max(self.nnodes, 1)
            self.act = torch.zeros(nn * 2 * NH, dtype=torch.float32, device=dev)
            self.gout = torch.zeros(nn * NO, dtype=torch.float32, device=dev)
            self.delta = torch.zeros(nn * (NO + 2 * NH), dtype=torch.float32, device=dev)
            self.z = torch.zeros(max(self.n, 1), dtype=torch.float64, device=dev)
            self.Kz = torch.zeros(max(self.n, 1), dtype=torch.float64, device=dev)


class TrainingSystem:
    """One plate's reduced system with residual samples from the FP64 solver.

    ``samples`` is a (k, n) CUDA tensor of residuals r = f - K u_i taken along
    an FP64 block-Jacobi PCG run; ``weights`` are 1 / (e_i . r_i) with
    e_i = u* - u_i the FP64 error against the converged solution."""

    def __init__(self, pattern, vals, samples, weights):
        from .solver import Solver
        self.pattern = pattern
        self.vals = vals
        self.samples = samples
        self.weights = np.asarray(weights, dtype=np.float64)
        self.solver = Solver(pattern).setup(vals)
        self._ctx = {}

    def context(self, feature_set=0):
        """Device buffers (features of the given set) of this system."""
        if feature_set not in self._ctx:
            self._ctx[feature_set] = _Ctx(self.solver, feature_set)
        return self._ctx[feature_set]

    @property
    def ctx(self):
        return self.context(0)


def make_training_system(pattern, vals, f, npairs=32, tol=1e-11, pair_tol=1e-7, stride=None):
    """Residual/error pairs of one system generated by the FP64 solver: the
    solution u* to ``tol``, then iterates u_i spaced evenly along a run to
    ``pair_tol`` (r_i = f - K u_i, e_i = u* - u_i)."""
    from .solver import Solver
    torch = _lib.torch_mod()
    s = Solver(pattern).setup(vals)
    fr = _lib.to_device(f, np.float64)
    ustar, st = s.solve(fr, tol=tol, check_every=50)
    if st['status'] != 'converged':
        raise RuntimeError('reference solve did not converge: %s' % st)
    if stride is None:
        _, stp = s.solve(fr, tol=pair_tol, check_every=50)
        stride = max(2, stp['iterations'] // (npairs + 1))
    u = torch.zeros_like(fr)
    R, w = [], []
    for _ in range(npairs):
        u, sti = s.solve(fr, u0=u, tol=1e-300, maxiter=stride, check_every=stride)
        r = fr - pattern.spmv(vals, u)
        e = ustar - u
        er = float(torch.dot(e, r))
        if not er > 0:
            break
        R.append(r)
        w.append(1. / er)
    samples = torch.stack(R) if R else torch.zeros((0, pattern.nrows), dtype=torch.float64, device=fr.device)
    return TrainingSystem(pattern, vals, samples, w)


class LearnedPC:
    """Per-node MLP block correction (weights on the GPU, FP32)."""

    def __init__(self, weights=None, seed=0, out_scale=0.1, mode=1, feature_set=0):
        torch = _lib.torch_mod()
        dev = _lib.device()
        W = init_weights(seed) if weights is None else np.asarray(weights, dtype=np.float32)
        if W.size != NW:
            raise ValueError('expected %d weights' % NW)
        self.W = torch.from_numpy(W.copy()).to(dev)
        self.out_scale = float(out_scale)
        # loss: 0 = energy error of z itself, 1 = after the optimal step along
        # z (scale-invariant, as CG is)
        self.mode = int(mode)
        # inputs: 0 = 35 features (scaled off-diagonals, log scales, free
        # mask, neighbour norms); 1 = 29 features (the 21 entries of the
        # normalised diagonal block and 8 neighbour-block norms)
        self.feature_set = int(feature_set)
        self.m = torch.zeros_like(self.W)
        self.v = torch.zeros_like(self.W)
        self.grad = torch.zeros_like(self.W)
        self.loss = torch.zeros(3, dtype=torch.float64, device=dev)  # [0] loss, [1..2] scratch
        self.step = 0
        self.history = []

    def weights(self):
        return self.W.cpu().numpy()

    def _forward_blocks(self, ctx, train):
        lib = _lib.load()
        sp = _lib.stream_ptr()
        act = None
        if train:
            ctx.train_buffers()
            act = ctx.act
        rc = lib.fe3d_lpc_forward(ctx.nnodes, _lib.ptr(ctx.feat), _lib.ptr(self.W), _lib.ptr(ctx.out),
                                  _lib.ptr(act), sp)
        _lib.check(rc, 'fe3d_lpc_forward')
        rc = lib.fe3d_lpc_blocks(ctx.solver._h, _lib.ptr(ctx.sdiag), _lib.ptr(ctx.out), self.out_scale,
                                 _lib.ptr(ctx.blocks), sp)
        _lib.check(rc, 'fe3d_lpc_blocks')
        nfb = c_int()
        rc = lib.fe3d_solver_set_blocks(ctx.solver._h, _lib.ptr(ctx.blocks), _lib.ptr(ctx.fallback),
                                        ctypes.byref(nfb), sp)
        _lib.check(rc, 'fe3d_solver_set_blocks')
        return nfb.value

    def install(self, solver, ctx=None):
        """Replace the solver's block-Jacobi blocks by the learned ones;
        returns the number of nodes that fell back to block Jacobi."""
        ctx = ctx or _Ctx(solver, self.feature_set)
        return self._forward_blocks(ctx, train=False)

    def loss_grad(self, system, idx):
        """Loss over the samples idx at the current weights; fills self.grad."""
        lib = _lib.load()
        sp = _lib.stream_ptr()
        ctx = system.context(self.feature_set)
        self._forward_blocks(ctx, train=True)
        ctx.gout.zero_()
        self.loss.zero_()
        pat = system.pattern
        for i in idx:
            r = system.samples[i]
            rc = lib.fe3d_lpc_apply(ctx.solver._h, _lib.ptr(r), _lib.ptr(ctx.z), sp)
            _lib.check(rc, 'fe3d_lpc_apply')
            pat.spmv(system.vals, ctx.z, ctx.Kz)
            rc = lib.fe3d_lpc_loss_grad(ctx.solver._h, _lib.ptr(ctx.sdiag), _lib.ptr(r), _lib.ptr(ctx.z),
                                        _lib.ptr(ctx.Kz), _lib.ptr(ctx.fallback), float(system.weights[i]),
                                        1. / len(idx), self.out_scale, self.mode, _lib.ptr(ctx.gout),
                                        _lib.ptr(self.loss), sp)
            _lib.check(rc, 'fe3d_lpc_loss_grad')
        self.grad.zero_()
        rc = lib.fe3d_lpc_backward(ctx.nnodes, _lib.ptr(ctx.feat), _lib.ptr(self.W), _lib.ptr(ctx.act),
                                   _lib.ptr(ctx.gout), _lib.ptr(ctx.delta), _lib.ptr(self.grad), sp)
        _lib.check(rc, 'fe3d_lpc_backward')
        return self.loss[0]

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        lib = _lib.load()
        self.step += 1
        rc = lib.fe3d_lpc_adam(NW, _lib.ptr(self.W), _lib.ptr(self.grad), _lib.ptr(self.m), _lib.ptr(self.v),
                               lr, beta1, beta2, eps, self.step, _lib.stream_ptr())
        _lib.check(rc, 'fe3d_lpc_adam')

    def objective(self, loss):
        """Relative squared energy error of the preconditioned residual."""
        return float(loss) if self.mode == 1 else 1. + float(loss)

    def evaluate(self, systems):
        """Mean relative squared energy error over all samples (every
        loss_grad call installs the current blocks first)."""
        vals = []
        for s in systems:
            if len(s.samples) == 0:
                continue
            vals.append(self.objective(self.loss_grad(s, range(len(s.samples))).item()))
        return float(np.mean(vals)) if vals else float('nan')

    def train(self, systems, steps=1000, batch=8, lr=1e-3, seed=0, log_every=50):
        """Adam on the mean loss of random sample batches, cycling over the
        systems; keeps (step, loss) in self.history."""
        rng = np.random.default_rng(seed)
        systems = [s for s in systems if len(s.samples)]
        for it in range(steps):
            s = systems[it % len(systems)]
            idx = rng.choice(len(s.samples), size=min(batch, len(s.samples)), replace=False)
            loss = self.loss_grad(s, idx)
            self.adam(lr)
            if log_every and it % log_every == 0:
                self.history.append((it, self.objective(loss.item())))
        return self.history

    def save(self, path):
        np.savez(path, W=self.weights(), out_scale=self.out_scale, mode=self.mode, feature_set=self.feature_set)

    @classmethod
    def load(cls, path):
        d = np.load(path)
        fs = int(d['feature_set']) if 'feature_set' in d else 0
        return cls(weights=d['W'], out_scale=float(d['out_scale']), mode=int(d['mode']), feature_set=fs)


def install_blocks(solver, blocks):
    """Install caller-given preconditioner blocks (device, 36 doubles per node,
    row-major over the node's free DOFs, zero padded) into a solver; returns
    the number of nodes that fell back to block Jacobi."""
    lib = _lib.load()
    torch = _lib.torch_mod()
    b = _lib.to_device(blocks, np.float64).reshape(-1).contiguous()
    nn = (solver.pattern.N + 5) // 6
    if b.numel() != 36 * nn:
        raise ValueError('expected 36 values per node')
    fb = torch.zeros(max(nn, 1), dtype=torch.int8, device=b.device)
    nfb = c_int()
    rc = lib.fe3d_solver_set_blocks(solver._h, _lib.ptr(b), _lib.ptr(fb), ctypes.byref(nfb), _lib.stream_ptr())
    _lib.check(rc, 'fe3d_solver_set_blocks')
    return nfb.value
