"""CPU restatement (NumPy) of the learned block preconditioner, for checking the device kernels: the edge network's
forward pass and its parameter gradients, the preconditioner's application and the training loss.

Test infrastructure only: tests/ alone imports this module, as the oracle of pcbqs_gb300_learned_* (the product
path runs those kernels, never this).

    M^-1 x = y - sum_e g_e D_b^-1 A_bc y_c,  y = D^-1 x        (edges e = (b <- c), blocks of bs unknowns)
    g_e    = w2 . tanh(W1 phi_e + b1) + b2
    loss   = |A M^-1 Z - Z|_F^2 / |Z|_F^2                        (Z the probe columns)
"""
import numpy as np


def unpack(params, nfeat, nhidden):
    h, f = nhidden, nfeat
    W1 = params[:h * f].reshape(h, f)
    b1 = params[h * f:h * f + h]
    w2 = params[h * f + h:h * f + 2 * h]
    b2 = params[h * f + 2 * h]
    return W1, b1, w2, b2


def forward(phi, params, nhidden):
    """(hidden (nedge, h), gains (nedge,))."""
    W1, b1, w2, b2 = unpack(params, phi.shape[1], nhidden)
    hidden = np.tanh(phi @ W1.T + b1)
    return hidden, hidden @ w2 + b2


def backward(phi, params, nhidden, hidden, dgains):
    """dL/dparams for dL/dgains."""
    W1, b1, w2, b2 = unpack(params, phi.shape[1], nhidden)
    dpre = dgains[:, None] * w2[None, :] * (1 - hidden ** 2)          # (nedge, h)
    return np.concatenate([(dpre.T @ phi).ravel(), dpre.sum(0), hidden.T @ dgains, [dgains.sum()]])


def apply(n, bs, eptr, ecol, dinv, E, gains, X):
    """M^-1 X (X (n, k) complex) and the correction vectors u (nedge, bs, k)."""
    nblk = len(eptr) - 1
    pad = nblk * bs
    Xp = np.zeros((pad, X.shape[1]), complex)
    Xp[:n] = X
    Y = np.einsum('bij,bjk->bik', dinv, Xp.reshape(nblk, bs, -1))
    out = Y.copy()
    U = np.zeros((len(ecol), bs, X.shape[1]), complex)
    for b in range(nblk):
        for e in range(eptr[b], eptr[b + 1]):
            U[e] = dinv[b] @ (E[e] @ Y[ecol[e]])
            if gains is not None:
                out[b] -= gains[e] * U[e]
    return out.reshape(pad, -1)[:n], U


def loss_and_gains_gradient(A, bs, eptr, ecol, dinv, E, gains, Z):
    """(loss, dloss/dgains) of |A M^-1 Z - Z|^2 / |Z|^2."""
    n = A.shape[0]
    X, U = apply(n, bs, eptr, ecol, dinv, E, gains, Z)
    R = A @ X - Z
    zz = float(np.vdot(Z, Z).real)
    S = A.conj().T @ R
    nblk = len(eptr) - 1
    Sp = np.zeros((nblk * bs, Z.shape[1]), complex)
    Sp[:n] = S
    Sb = Sp.reshape(nblk, bs, -1)
    dots = np.zeros(len(ecol))
    for b in range(nblk):
        for e in range(eptr[b], eptr[b + 1]):
            dots[e] = float(np.sum(Sb[b].real * U[e].real + Sb[b].imag * U[e].imag))
    return float(np.vdot(R, R).real) / zz, -2 * dots / zz
