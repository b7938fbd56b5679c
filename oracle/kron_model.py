"""Independent cross-check of the oracle: Zeeman-basis Liouville model.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).

Builds the secular NMR Liouvillian of a small spin system directly from
Hilbert-space spin operators (Kronecker products of single-spin matrices),
with interaction tensors rotated by the Euler angles as Cartesian matrices.
It shares no code with the spherical-tensor path (no product tables, no
superop.m restatement, no Wigner matrices), so agreement of full-basis FIDs
pins the basis, normalisation, operator and relaxation conventions of the
oracle.  Only the direction of the rotation is a convention choice; it is the
one that makes R = euler2dcm(alpha,beta,gamma) act on the interaction tensors
as R A R^T (an active rotation of the molecule).
"""
from __future__ import annotations

import math

import numpy as np
import scipy.linalg as sla

from .spinach_ref import ISOTOPES, euler2dcm, pauli


def _embed(op, s, mults):
    out = np.eye(1, dtype=complex)
    for i, m in enumerate(mults):
        out = np.kron(out, op if i == s else np.eye(m))
    return out


class KronModel:
    def __init__(self, ss):
        """``ss`` is an oracle SpinSystem after create() (NMR isotopes only)."""
        self.ss = ss
        self.mults = [int(m) for m in ss.mults]
        self.ops = []
        for s, m in enumerate(self.mults):
            P = pauli(m)
            self.ops.append({k: _embed(P[k], s, self.mults) for k in ('x', 'y', 'z', 'p', 'm')})
        self.dim = int(np.prod(self.mults))

    def hamiltonian(self, angles):
        """Secular NMR Hamiltonian (rad/s) in the rotating frame at one orientation."""
        ss = self.ss
        Rm = euler2dcm(*angles)
        H = np.zeros((self.dim, self.dim), complex)
        for s in range(ss.nspins):
            Z = Rm @ ss.zeeman[s] @ Rm.T
            H += (Z[2, 2] - ss.basefrqs[s]) * self.ops[s]['z']
        for (a, b), A in ss.coupling.items():
            Ar = Rm @ A @ Rm.T
            if a == b:
                # quadratic coupling L.A.L, secular part (A_zz/2)(3 Lz^2 - L^2)
                Lz = self.ops[a]['z']
                s_ = (self.mults[a] - 1) / 2
                H += (Ar[2, 2] / 2) * (3 * Lz @ Lz - s_ * (s_ + 1) * np.eye(self.dim))
                continue
            iso = np.trace(A) / 3
            Oa, Ob = self.ops[a], self.ops[b]
            zz = Oa['z'] @ Ob['z']
            flip = Oa['x'] @ Ob['x'] + Oa['y'] @ Ob['y']
            if ss.isotopes[a] == ss.isotopes[b]:
                H += iso * (zz + flip) + (Ar[2, 2] - iso) * (zz - flip / 2)
            else:
                H += Ar[2, 2] * zz
        return H

    def relaxation(self):
        """T1/T2 superoperator: each spin's longitudinal part decays at R1 and its
        transverse part at R2, summed over spins."""
        d = self.dim
        Rl = np.zeros((d * d, d * d), complex)
        if 't1_t2' not in self.ss.theories:
            return Rl
        for s, m in enumerate(self.mults):
            if m != 2:
                raise ValueError('kron relaxation model covers spin-1/2 only')
            # single-spin superoperator on row-major vec(rho_s)
            rs = np.zeros((4, 4))
            r1, r2 = self.ss.r1[s], self.ss.r2[s]
            # basis |a><a|, |a><b|, |b><a|, |b><b|: populations relax towards their mean
            rs[0, 0] = rs[3, 3] = -r1 / 2
            rs[0, 3] = rs[3, 0] = r1 / 2
            rs[1, 1] = rs[2, 2] = -r2
            # embed: vec over the whole space, act on spin s
            left = int(np.prod(self.mults[:s])) if s else 1
            right = int(np.prod(self.mults[s + 1:])) if s + 1 < len(self.mults) else 1
            for i0 in range(2):
                for j0 in range(2):
                    for i1 in range(2):
                        for j1 in range(2):
                            v = rs[2 * i1 + j1, 2 * i0 + j0]
                            if v == 0:
                                continue
                            for a in range(left):
                                for b in range(right):
                                    for a2 in range(left):
                                        for b2 in range(right):
                                            row = ((a * 2 + i1) * right + b) * d + (a2 * 2 + j1) * right + b2
                                            col = ((a * 2 + i0) * right + b) * d + (a2 * 2 + j0) * right + b2
                                            Rl[row, col] += v
        return Rl

    def spin_op(self, op, isotope):
        key = {'Lx': 'x', 'Ly': 'y', 'Lz': 'z', 'L+': 'p', 'L-': 'm'}[op]
        out = np.zeros((self.dim, self.dim), complex)
        for s, iso in enumerate(self.ss.isotopes):
            if iso == isotope:
                out += self.ops[s][key]
        return out

    def fid(self, angles, rho0, coil, dt, nsteps):
        """fid(n) = Tr(coil^dagger rho(n dt)), rho evolving under -i[H,.] + R."""
        H = self.hamiltonian(angles)
        I = np.eye(self.dim)
        L = np.kron(H, I) - np.kron(I, H.T) + 1j * self.relaxation()
        P = sla.expm(-1j * dt * L)
        r = rho0.reshape(-1).astype(complex)
        c = coil.reshape(-1)
        out = np.zeros(nsteps + 1, complex)
        for n in range(nsteps + 1):
            out[n] = np.vdot(c, r)
            r = P @ r
        return out

    def cpmg(self, angles, rho0, coil, pulse_op, dt, npoints, nloops):
        """CPMG echo train with hard pulses U rho U^dagger, U = exp(-1i theta
        pulse_op) (Hilbert space), theta = pi/2 first and pi in every loop;
        segments of npoints-1 and 2*npoints-1 steps, each starting from the
        pulsed last state of the one before."""
        H = self.hamiltonian(angles)
        I = np.eye(self.dim)
        L = np.kron(H, I) - np.kron(I, H.T) + 1j * self.relaxation()
        P = sla.expm(-1j * dt * L)
        c = coil.reshape(-1)

        def pulse(r, theta):
            U = sla.expm(-1j * theta * pulse_op)
            return (U @ r.reshape(self.dim, self.dim) @ U.conj().T).reshape(-1)

        r = pulse(rho0.reshape(-1).astype(complex), np.pi / 2)
        out = []
        for seg in range(nloops + 1):
            n = npoints - 1 if seg == 0 else 2 * npoints - 1
            if seg:
                r = pulse(r, np.pi)
            for k in range(n + 1):
                out.append(np.vdot(c, r))
                if k < n:
                    r = P @ r
        return np.array(out)

    def eseem(self, angles, rho0, coil, pulse_op, timestep, npoints, first_angle=np.pi / 2):
        """Two-pulse echo: U rho U^dagger pulses (first_angle, 90 degrees by
        default, then 180 degrees), point n after n steps of timestep/2 on
        each side of the 180-degree pulse."""
        H = self.hamiltonian(angles)
        I = np.eye(self.dim)
        L = np.kron(H, I) - np.kron(I, H.T) + 1j * self.relaxation()
        P = sla.expm(-1j * (timestep / 2) * L)

        def pulse(r, theta):
            U = sla.expm(-1j * theta * pulse_op)
            return (U @ r.reshape(self.dim, self.dim) @ U.conj().T).reshape(-1)

        r = pulse(rho0.reshape(-1).astype(complex), first_angle)
        c = coil.reshape(-1)
        out = []
        for n in range(npoints):
            x = pulse(r, np.pi)
            for _ in range(n):
                x = P @ x
            out.append(np.vdot(c, x))
            r = P @ r
        return np.array(out)

    def deer_3p(self, angles, rho0, coil, ex_prob, ex_pump, stepsize, nsteps):
        """Three-pulse DEER with hard pulses U rho U^dagger: probe 90 degrees,
        j steps, pump 180 degrees, nsteps-j steps, probe 180 degrees, nsteps
        steps; point j is <coil, state> (not normalised), j = 0..nsteps."""
        H = self.hamiltonian(angles)
        I = np.eye(self.dim)
        L = np.kron(H, I) - np.kron(I, H.T) + 1j * self.relaxation()
        P = sla.expm(-1j * stepsize * L)

        def pulse(r, op, theta):
            U = sla.expm(-1j * theta * op)
            return (U @ r.reshape(self.dim, self.dim) @ U.conj().T).reshape(-1)

        r = pulse(rho0.reshape(-1).astype(complex), ex_prob, np.pi / 2)
        c = coil.reshape(-1)
        out = []
        for j in range(nsteps + 1):
            x = pulse(r, ex_pump, np.pi)
            for _ in range(nsteps - j):
                x = P @ x
            x = pulse(x, ex_prob, np.pi)
            for _ in range(nsteps):
                x = P @ x
            out.append(np.vdot(c, x))
            r = P @ r
        return np.array(out)


def gamma_of(isotope):
    return ISOTOPES[isotope][1]


__all__ = ['KronModel', 'gamma_of', 'math']
