"""Magic-angle spinning in the Fokker-Planck formalism (kernel/contexts/singlerot.m).

The single-rotor context samples the rotor phase on N = 2*max_rank+1 points
and couples them with the Fourier collocation derivative: per orientation

    L = blkdiag(H_1 .. H_N) + 1i*M + 1i*kron(eye(N), R),
    H_n = I + sum_{r,k,m} D_comp^{(n)}(k,m) Q{r}{k,m},
    D_comp^{(n)} = D_lab2rot * D_rotor(phi_n) * D_mol2rot(alpha, beta, gamma),
    M = 2*pi*rate*kron(d/dphi, eye(dim))                    (singlerot.m:259-306)

Since D_comp^{(n)}(k,m) = sum_j A^{(n)}(k,j) D_mol2rot(j,m) with the
orientation-independent A^{(n)} = D_lab2rot * D_rotor(phi_n), the whole
Fokker-Planck Liouvillian is again I' + sum_{r,j,m} D^r_{jm}(Omega) Q'{r}{j,m}
with

    I' = kron(eye(N), I) + 1i*M,
    Q'{r}{j,m} = blkdiag_n( sum_k A^{(n)}(k,j) Q{r}{k,m} ),

which is exactly the form the engine's upload takes: the rotor-space problem
runs through the same kernels, orientations and powder sum unchanged.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp


def wigner_d(l: int, alpha: float, beta: float, gamma: float) -> np.ndarray:
    """Wigner D^l(alpha, beta, gamma), rows and columns in descending
    projection l..-l, D(m', m) = exp(-1i m' alpha) d(m', m)(beta) exp(-1i m gamma)
    (the convention of kernel/utilities/wigner.m); d from Wigner's sum formula."""
    ms = np.arange(l, -l - 1, -1)
    c, s = math.cos(beta / 2), math.sin(beta / 2)
    f = math.factorial
    D = np.zeros((2 * l + 1, 2 * l + 1), complex)
    for i, mp in enumerate(ms):
        for j, m in enumerate(ms):
            pref = math.sqrt(f(l + mp) * f(l - mp) * f(l + m) * f(l - m))
            tot = 0.0
            for k in range(max(0, m - mp), min(l + m, l - mp) + 1):
                num = (-1) ** (mp - m + k)
                den = f(l + m - k) * f(k) * f(mp - m + k) * f(l - mp - k)
                tot += num / den * c ** (2 * l + m - mp - 2 * k) * s ** (mp - m + 2 * k)
            D[i, j] = np.exp(-1j * mp * alpha) * pref * tot * np.exp(-1j * m * gamma)
    return D


def fourier_derivative(n: int):
    """Rotor phases 2*pi*k/n and the first-derivative Fourier collocation
    matrix on them (kernel/derivatives/fourdif.m, m = 1): entry (j, k) is
    (-1)^(j-k)/2 * cot((j-k) h/2) for even n and csc((j-k) h/2) for odd n,
    h = 2*pi/n, zero on the diagonal."""
    x = 2 * np.pi * np.arange(n) / n
    h = 2 * np.pi / n
    d = np.arange(n)[:, None] - np.arange(n)[None, :]
    D = np.zeros((n, n))
    off = d != 0
    arg = d[off] * h / 2
    trig = 1 / np.tan(arg) if n % 2 == 0 else 1 / np.sin(arg)
    D[off] = 0.5 * np.where(d[off] % 2 == 0, 1.0, -1.0) * trig
    return x, D


def rotor_axis_angles(axis) -> tuple:
    """Lab-frame rotor direction as (phi, theta): azimuth and polar angle
    (singlerot.m:159-163, MATLAB cart2sph with theta = pi/2 - elevation)."""
    x, y, z = (float(v) for v in axis)
    phi = math.atan2(y, x)
    elevation = math.atan2(z, math.hypot(x, y))
    return phi, math.pi / 2 - elevation


def fokker_planck(I, terms: dict, R, rho0, coil, max_rank: int, rate: float, axis,
                  single_crystal: bool = False):
    """The single-rotor Fokker-Planck system in the engine's upload form.

    ``terms`` maps (rank, k, m) with 0-based k, m to Q{rank}{k,m}.  Returns
    ``(I', terms', R', rho0', coil')``: rho0' = kron(ones(N)/N, rho0) for a
    powder (rotor phase averaging), kron(e_1, rho0) for a single crystal, and
    coil' = kron(ones(N), coil) (singlerot.m:197-215)."""
    if max_rank < 0 or int(max_rank) != max_rank:
        raise ValueError('max_rank must be a non-negative integer')
    N = 2 * int(max_rank) + 1
    dim = I.shape[0]
    phases, Dfd = fourier_derivative(N)
    phi, theta = rotor_axis_angles(axis)
    eye_n = sp.identity(N, format='csr')
    M = 2 * np.pi * rate * sp.kron(sp.csr_matrix(Dfd), sp.identity(dim), format='csr')
    I_fp = (sp.kron(eye_n, sp.csr_matrix(I)) + 1j * M).tocsr()
    ranks = sorted({key[0] for key in terms})
    A = {r: [wigner_d(r, phi, theta, 0.0) @ wigner_d(r, 0.0, 0.0, p) for p in phases] for r in ranks}
    out = {}
    for r in ranks:
        for j in range(2 * r + 1):
            for m in range(2 * r + 1):
                blocks = []
                for n in range(N):
                    acc = None
                    for k in range(2 * r + 1):
                        Q = terms.get((r, k, m))
                        c = A[r][n][k, j]
                        if Q is None or c == 0:
                            continue
                        acc = c * Q if acc is None else acc + c * Q
                    blocks.append(sp.csr_matrix((dim, dim), dtype=complex) if acc is None else sp.csr_matrix(acc))
                B = sp.block_diag(blocks, format='csr')
                B.eliminate_zeros()
                if B.nnz:
                    out[(r, j, m)] = B
    R_fp = None if R is None else sp.kron(eye_n, sp.csr_matrix(R), format='csr')
    space = np.zeros(N)
    if single_crystal:
        space[0] = 1.0
    else:
        space[:] = 1.0 / N
    rho0_fp = np.kron(space, np.asarray(rho0, complex))
    coil_fp = np.kron(np.ones(N), np.asarray(coil, complex))
    return I_fp, out, R_fp, rho0_fp, coil_fp


def floquet_system(I, terms: dict, R, rho0, coil, max_rank: int, rate: float, axis):
    """Floquet MAS (kernel/contexts/floquet.m:94-186) in the engine's upload
    form.  The Floquet Liouvillian of an orientation is

        F = sum_h kron(S_h, T_h(Omega)) + M,  M = 2*pi*rate*kron(diag(-N..N), 1),

    S_h the shift by h in the (2N+1)-dimensional Fourier space, T_0 containing
    I, and T_{n-r} (n = 0..2r) += sum_{k,m} D(k,m) Q{r}{k,m} with
    D = D_lab2rot P_n D_rot2lab (D_lab2rot D_mol2rot(Omega) D_rot2lab).  With
    A_n = D_lab2rot P_n D_rot2lab D_lab2rot and B = D_rot2lab,
    D(k,m) = sum_{j,l} A_n(k,j) D_mol2rot(j,l) B(l,m): the orientation enters
    through D_mol2rot alone, so F = I' + sum D_mol2rot(j,l) Q'{r}{j,l}.  The
    states live in the zeroth Fourier component (floquet.m:142-148)."""
    if max_rank < 0 or int(max_rank) != max_rank:
        raise ValueError('max_rank must be a non-negative integer')
    ranks = sorted({key[0] for key in terms})
    max_int = max(ranks + [2])
    if max_int > max_rank:
        raise ValueError('max_rank must be at least the highest interaction rank')
    N = 2 * int(max_rank) + 1
    dim = I.shape[0]
    phi, theta = rotor_axis_angles(axis)
    def shift(d):
        return sp.diags(np.ones(N - abs(d)), d, shape=(N, N), format='csr')
    M = 2 * np.pi * rate * sp.kron(sp.diags(np.arange(-max_rank, max_rank + 1, dtype=float)), sp.identity(dim))
    I_f = (sp.kron(sp.identity(N), sp.csr_matrix(I)) + M).tocsr()
    out = {}
    for r in ranks:
        L2R = wigner_d(r, phi, theta, 0.0)
        R2L = L2R.conj().T
        A = []
        for n in range(2 * r + 1):
            Pn = np.zeros((2 * r + 1, 2 * r + 1))
            Pn[n, n] = 1.0
            A.append(L2R @ Pn @ R2L @ L2R)
        for j in range(2 * r + 1):
            for l in range(2 * r + 1):
                acc = None
                for n in range(2 * r + 1):
                    blk = None
                    for k in range(2 * r + 1):
                        for m in range(2 * r + 1):
                            Q = terms.get((r, k, m))
                            c = A[n][k, j] * R2L[l, m]
                            if Q is None or abs(c) == 0:
                                continue
                            blk = c * Q if blk is None else blk + c * Q
                    if blk is None:
                        continue
                    term = sp.kron(shift(n - r), sp.csr_matrix(blk))
                    acc = term if acc is None else acc + term
                if acc is not None:
                    acc = sp.csr_matrix(acc)
                    acc.eliminate_zeros()
                    if acc.nnz:
                        out[(r, j, l)] = acc
    R_f = None if R is None else sp.kron(sp.identity(N), sp.csr_matrix(R), format='csr')
    centre = np.zeros(N)
    centre[N // 2] = 1.0
    return I_f, out, R_f, np.kron(centre, np.asarray(rho0, complex)), np.kron(centre, np.asarray(coil, complex))
