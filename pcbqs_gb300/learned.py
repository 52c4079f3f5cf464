"""A learned block preconditioner for the PEEC loop/tree systems, trained on the GPU by this library's own kernels.

    systems = [block_system_of(PeecModel(board).assemble(), f) for board, f in ...]
    params, history = train(systems)                 # the edge network's 129 parameters
    its_bj, its_learned = compare(system, params)    # GMRES steps: block-Jacobi alone, and with the learned gains

The preconditioner is block-Jacobi over the clustered blocks of `bs` unknowns plus, for the `per_block` most
strongly coupled blocks c of every block b, a Neumann-type correction -g_e D_b^-1 A_bc y_c whose gain g_e a small
edge-level network (one hidden layer of 16 tanh units) predicts from the pair's features: its coupling strength both
ways, the size of the correction, the share of loop unknowns on each side and the frequency. All gains zero is block
Jacobi, where the training starts; the training minimises the preconditioned residual |A M^-1 Z - Z|^2 / |Z|^2 of
random probe columns Z, relative to block-Jacobi's, averaged over the systems, with Adam. The forward and backward
passes, the preconditioner and the gradient dots are the CUDA kernels of csrc/learned.cu (pcbqs_gb300_learned_*);
the dense products with A and A^H are cuBLAS. Training data: the systems of seeded random boards
(tests/golden/train_*.npz) at random frequencies; the boards named in the tests are held out.

    python -m pcbqs_gb300.learned train [out.npz [l2]]    # train on the random boards and save the parameters
"""
import ctypes
import sys
from dataclasses import dataclass
from pathlib import Path

import numpy as np
import torch

from . import _lib

NFEAT, NHIDDEN = 6, 16
NPARAMS = NHIDDEN * NFEAT + 2 * NHIDDEN + 1
PARAMS = Path(__file__).resolve().parent / 'learned_params.npz'


def _stream(device=None):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


@dataclass
class BlockSystem:
    """A dense system in blocks of `bs` unknowns with its edge list, blocks and edge features (device arrays)."""
    A: torch.Tensor              # (n, n) complex128, row-major
    bs: int
    dinv: torch.Tensor           # (nblk, bs, bs) complex128: inverted diagonal blocks (identity-padded)
    eptr: torch.Tensor           # (nblk + 1,) int64: edges grouped by destination block
    ecol: torch.Tensor           # (nedge,) int32: source block of each edge
    E: torch.Tensor              # (nedge, bs, bs) complex128: the coupling blocks A_bc (zero-padded)
    phi: torch.Tensor            # (nedge, NFEAT) float64
    name: str = ''

    @property
    def n(self):
        return self.A.shape[0]

    @property
    def nblk(self):
        return len(self.eptr) - 1

    @property
    def nedge(self):
        return len(self.ecol)


def block_system(A, is_loop, freq, bs=32, per_block=6, name=''):
    """Blocks, edges and features of the dense complex system A (n, n) (its unknowns in the clustered order;
    is_loop (n,) marks the loop unknowns) at frequency `freq` (Hz)."""
    dev = A.device
    n = A.shape[0]
    nblk = (n + bs - 1) // bs
    pad = nblk * bs
    Ap = torch.zeros((pad, pad), dtype=torch.complex128, device=dev)
    Ap[:n, :n] = A
    if pad > n:
        idx = torch.arange(n, pad, device=dev)
        Ap[idx, idx] = 1
    blocks = Ap.reshape(nblk, bs, nblk, bs).permute(0, 2, 1, 3)
    diag = torch.arange(nblk, device=dev)
    # row-major like every array the kernels take (the batched inverse comes back column-major per block)
    dinv = torch.linalg.inv(blocks[diag, diag].contiguous()).contiguous()
    norms = torch.linalg.norm(blocks, dim=(2, 3))
    dn = torch.diagonal(norms).clamp_min(1e-300)
    rho = norms / torch.sqrt(dn[:, None] * dn[None, :])
    rho.fill_diagonal_(0)
    m = min(per_block, max(nblk - 1, 0))
    if m:
        vals, cols = torch.topk(rho, m, dim=1)
        keep = vals > 1e-6
        b_idx = diag[:, None].expand(nblk, m)[keep]
        c_idx = cols[keep]
        order = torch.argsort(b_idx * nblk + c_idx)
        b_idx, c_idx = b_idx[order], c_idx[order]
    else:
        b_idx = c_idx = torch.zeros(0, dtype=torch.int64, device=dev)
    E = blocks[b_idx, c_idx].contiguous()
    eptr = torch.zeros(nblk + 1, dtype=torch.int64, device=dev)
    eptr[1:] = torch.cumsum(torch.bincount(b_idx, minlength=nblk), 0)
    corr = torch.linalg.norm(dinv[b_idx] @ E, dim=(1, 2)) / np.sqrt(bs)
    loop = torch.zeros(pad, dtype=torch.float64, device=dev)
    loop[:n] = torch.as_tensor(np.asarray(is_loop, float), device=dev)
    frac = loop.reshape(nblk, bs).mean(1)
    lg = lambda t: torch.log10(t.clamp_min(1e-300))
    phi = torch.stack([lg(rho[b_idx, c_idx]), lg(corr), lg(rho[c_idx, b_idx]), frac[b_idx], frac[c_idx],
                       torch.full_like(corr, np.log10(freq / 1e6) / 3)], dim=1).contiguous()
    return BlockSystem(A.contiguous(), bs, dinv, eptr, c_idx.to(torch.int32).contiguous(), E, phi, name)


def peec_system(model, freq, chunk=512):
    """The dense loop/tree system of a PeecModel (assembled) at `freq` (Hz), column by column from the operator:
    (A (n, n) complex128 on the device, is_loop (n,))."""
    lib = _lib.load()
    handle, _ = model._operator(np.array([2 * np.pi * freq]))
    n = model.n
    A = torch.empty((n, n), dtype=torch.complex128, device=model.device)
    try:
        for j0 in range(0, n, chunk):
            m = min(chunk, n - j0)
            X = torch.zeros((n, m), dtype=torch.complex128, device=model.device)
            X[torch.arange(j0, j0 + m), torch.arange(m)] = 1
            Y = torch.empty_like(X)
            sys_ = np.zeros(m, np.int32)
            _lib.check(lib.pcbqs_gb300_peec_apply(handle, m, _lib.ptr(sys_, ctypes.c_int32), X.data_ptr(),
                                                  Y.data_ptr(), _stream(model.device)), lib)
            A[:, j0:j0 + m] = Y
    finally:
        lib.pcbqs_gb300_peec_destroy(handle)
    return A, model.is_tree == 0


def block_system_of(model, freq, **kw):
    A, is_loop = peec_system(model, freq)
    return block_system(A, is_loop, freq, **kw)


# ---- the device kernels ------------------------------------------------------------------------------------------

def forward(system, params):
    """(hidden (nedge, NHIDDEN), gains (nedge,)) of the edge network."""
    lib = _lib.load()
    dev = system.A.device
    hidden = torch.empty((max(system.nedge, 1), NHIDDEN), dtype=torch.float64, device=dev)
    gains = torch.empty(max(system.nedge, 1), dtype=torch.float64, device=dev)
    _lib.check(lib.pcbqs_gb300_learned_forward(system.nedge, NFEAT, NHIDDEN, system.phi.data_ptr(), params.data_ptr(),
                                               hidden.data_ptr(), gains.data_ptr(), _stream(dev)), lib)
    return hidden[:system.nedge], gains[:system.nedge]


def backward(system, params, hidden, dgains):
    lib = _lib.load()
    grad = torch.empty(NPARAMS, dtype=torch.float64, device=params.device)
    _lib.check(lib.pcbqs_gb300_learned_backward(system.nedge, NFEAT, NHIDDEN, system.phi.data_ptr(),
                                                params.data_ptr(), hidden.data_ptr(), dgains.data_ptr(),
                                                grad.data_ptr(), _stream(params.device)), lib)
    return grad


def apply(system, gains, X, corrections=False):
    """M^-1 X (n, k) complex128 (gains None: block-Jacobi), and the correction vectors (nedge, bs, k) if asked."""
    lib = _lib.load()
    X = X.contiguous()
    out = torch.empty_like(X)
    k = X.shape[1]
    U = torch.empty((max(system.nedge, 1), system.bs, k), dtype=torch.complex128, device=X.device) \
        if corrections else None
    _lib.check(lib.pcbqs_gb300_learned_apply(system.n, system.bs, system.nblk, system.eptr.data_ptr(),
                                             system.ecol.data_ptr(), system.dinv.data_ptr(), system.E.data_ptr(),
                                             gains.data_ptr() if gains is not None else None, k, X.data_ptr(),
                                             out.data_ptr(), U.data_ptr() if U is not None else None,
                                             _stream(X.device)), lib)
    return (out, U) if corrections else out


def loss_and_gradient(system, params, Z, l2=0.0):
    """(loss |A M^-1 Z - Z|^2 / |Z|^2, dloss/dparams) through the device kernels; l2 > 0 adds l2 mean(g^2) to
    the gradient (not to the loss reported)."""
    lib = _lib.load()
    hidden, gains = forward(system, params)
    X, U = apply(system, gains, Z, corrections=True)
    R = system.A @ X - Z
    zz = float(torch.vdot(Z.flatten(), Z.flatten()).real)
    S = (system.A.conj().T @ R).contiguous()
    dots = torch.empty(max(system.nedge, 1), dtype=torch.float64, device=Z.device)
    _lib.check(lib.pcbqs_gb300_learned_edge_dots(system.n, system.bs, system.nblk, system.eptr.data_ptr(), Z.shape[1],
                                                 S.data_ptr(), U.data_ptr(), dots.data_ptr(), _stream(Z.device)),
               lib)
    dgains = (-2 / zz) * dots[:system.nedge]
    if l2 and system.nedge:
        dgains = dgains + (2 * l2 / system.nedge) * gains
    loss = float(torch.vdot(R.flatten(), R.flatten()).real) / zz
    return loss, backward(system, params, hidden, dgains.contiguous())


def initial_params(seed=0, device='cuda'):
    """Random first layer, zero output layer: every gain 0, block-Jacobi."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAMS)
    p[:NHIDDEN * NFEAT] = rng.normal(0, 0.5 / np.sqrt(NFEAT), NHIDDEN * NFEAT)
    return torch.as_tensor(p, device=device)


def probes(system, k=16, seed=0):
    g = torch.Generator(device=system.A.device).manual_seed(seed)
    shape = (system.n, k)
    return torch.complex(torch.randn(shape, dtype=torch.float64, device=system.A.device, generator=g),
                         torch.randn(shape, dtype=torch.float64, device=system.A.device, generator=g))


def train(systems, steps=300, lr=0.02, k=16, seed=0, l2=0.0, log=None):
    """Adam on the mean over systems of loss / block-Jacobi's loss (+ l2 times the mean squared gain, which keeps
    the corrections modest where the probes do not ask for them), fixed probes per system. Returns (params, history
    of the mean relative loss)."""
    dev = systems[0].A.device
    params = initial_params(seed, dev)
    Zs = [probes(s, k, seed + i) for i, s in enumerate(systems)]
    base = [loss_and_gradient(s, torch.zeros(NPARAMS, dtype=torch.float64, device=dev), Z)[0]
            for s, Z in zip(systems, Zs)]
    m = torch.zeros_like(params)
    v = torch.zeros_like(params)
    beta1, beta2, eps = 0.9, 0.999, 1e-12
    history = []
    for step in range(steps):
        grad = torch.zeros_like(params)
        total = 0.0
        for s, Z, b in zip(systems, Zs, base):
            loss, gr = loss_and_gradient(s, params, Z, l2 * b)
            total += loss / b
            grad += gr / b
        grad /= len(systems)
        history.append(total / len(systems))
        m = beta1 * m + (1 - beta1) * grad
        v = beta2 * v + (1 - beta2) * grad * grad
        mh = m / (1 - beta1 ** (step + 1))
        vh = v / (1 - beta2 ** (step + 1))
        params = params - lr * mh / (torch.sqrt(vh) + eps)
        if log and (step % 25 == 0 or step == steps - 1):
            log(f'step {step}: mean relative loss {history[-1]:.4f}')
    return params, history


def gmres(system, gains, b, tol=1e-8, maxiter=2000, restart=100):
    """(x, iterations per column, residuals) of A x = b by this library's GMRES, right-preconditioned by block
    Jacobi (gains None) or the learned preconditioner."""
    lib = _lib.load()
    b = b.contiguous()
    x = torch.zeros_like(b)
    k = b.shape[1]
    its, res = np.zeros(k, np.int32), np.zeros(k)
    status = lib.pcbqs_gb300_learned_gmres(system.n, system.A.data_ptr(), system.A.stride(0), k, b.data_ptr(),
                                           x.data_ptr(), tol, maxiter, restart, system.bs, system.nblk,
                                           system.eptr.data_ptr(), system.ecol.data_ptr(), system.dinv.data_ptr(),
                                           system.E.data_ptr(), gains.data_ptr() if gains is not None else None,
                                           _lib.ptr(its, ctypes.c_int32), _lib.ptr(res), _stream(b.device))
    if status not in (0, 5):
        _lib.check(status, lib)
    return x, its, res


def compare(system, params, k=4, seed=1):
    """GMRES steps per column to 1e-8 with block-Jacobi and with the learned gains, same right-hand sides."""
    b = probes(system, k, seed)
    _, its_bj, _ = gmres(system, None, b)
    _, gains = forward(system, params)
    _, its_l, res = gmres(system, gains, b)
    return its_bj, its_l, res


def save(params, path=PARAMS, **info):
    np.savez(path, params=params.cpu().numpy(), nfeat=NFEAT, nhidden=NHIDDEN, **info)


def load(path=PARAMS, device='cuda'):
    with np.load(path) as d:
        if int(d['nfeat']) != NFEAT or int(d['nhidden']) != NHIDDEN:
            raise ValueError('learned parameters of another network shape')
        return torch.as_tensor(d['params'], device=device)


TRAIN_BOARDS = tuple(f'train_{i}' for i in range(6))
TRAIN_FREQS = (1e5, 1e6, 1e7)


def training_systems(boards=TRAIN_BOARDS, freqs=TRAIN_FREQS, log=None):
    from .board import Board
    from .peec import PeecModel
    out = []
    for name in boards:
        model = PeecModel(Board.load(name)).assemble()
        for f in freqs:
            out.append(block_system_of(model, f, name=f'{name}@{f:g}'))
            if log:
                log(f'{name} at {f:g} Hz: n {out[-1].n}, {out[-1].nblk} blocks, {out[-1].nedge} edges')
    return out


def main(argv):
    if not argv or argv[0] != 'train':
        print(__doc__)
        return 2
    out = Path(argv[1]) if len(argv) > 1 else PARAMS
    l2 = float(argv[2]) if len(argv) > 2 else 0.0
    systems = training_systems(log=print)
    params, history = train(systems, l2=l2, log=print)
    save(params, out, history=np.asarray(history), boards=np.array(TRAIN_BOARDS), freqs=np.array(TRAIN_FREQS),
         l2=l2)
    print(f'saved {out}: relative loss {history[0]:.4f} -> {history[-1]:.4f}')
    return 0


if __name__ == '__main__':
    sys.exit(main(sys.argv[1:]))
