"""Seeded synthetic mid-run states for single-step parity cases (test infrastructure only).

A state is what ``ref_harness forces`` injects: perturbed current coordinates, nodal Current fields
and integration-point state.  Tensors are symmetric; for axisymmetric elements only the rr, zz, tt
and rz components are non-zero, as an axisymmetric run produces.  Deviatoric stress magnitudes are
drawn around the current yield stress so that both the elastic and the plastic branches of the
radial return are exercised.
"""

from __future__ import annotations

import numpy as np


def _sym(rng, shape, scale, two_d):
    t = rng.normal(scale=scale, size=shape + (3, 3))
    t = 0.5 * (t + np.swapaxes(t, -1, -2))
    if two_d:
        t[..., 0, 2] = t[..., 2, 0] = t[..., 1, 2] = t[..., 2, 1] = 0.0
    return t


def random_state(model, seed: int = 0, du_scale: float = 2e-3, dt: float = 1e-8):
    rng = np.random.default_rng(seed)
    m = model
    axi = m.etype == 0
    two_d = m.etype != 1
    dim, N, E, nip = m.dim, m.N, m.E, m.nip
    if getattr(m, "groups", None):
        # several element types (3D): per-IP arrays flat over every group's points, element order
        two_d = False
        E, nip = m.nIP_all, 1
    x = m.coords[m.conn]  # (E, nen, 3)
    h = float(np.min(np.linalg.norm(x[:, 1] - x[:, 0], axis=1)))
    coords = m.coords.copy()
    jit = rng.uniform(-0.04, 0.04, size=(N, dim)) * h
    if axi:  # keep nodes on the axis on it
        jit[m.coords[:, 0] == 0.0, 0] = 0.0
    coords[:, :dim] += jit
    du = np.zeros((N, 3))
    du[:, :dim] = rng.normal(scale=du_scale * h, size=(N, dim))
    if axi:
        du[m.coords[:, 0] == 0.0, 0] = 0.0
    v = np.zeros((N, 3))
    v[:, :dim] = rng.normal(scale=50.0, size=(N, dim))
    a = np.zeros((N, 3))
    a[:, :dim] = rng.normal(scale=1e8, size=(N, dim))
    disp = np.zeros((N, 3))
    disp[:, :dim] = rng.normal(scale=1e-4, size=(N, dim))

    evp = rng.uniform(1e-10, 0.4, size=(E, nip))
    evp[rng.uniform(size=(E, nip)) < 0.2] = 1e-10
    sig_y = m.A + m.B * evp ** m.n
    S = _sym(rng, (E, nip), 1.0, two_d)
    tr = np.trace(S, axis1=-2, axis2=-1)[..., None, None] / 3.0
    S = S - tr * np.eye(3)
    nrm = np.sqrt(1.5 * np.sum(S * S, axis=(-1, -2)))
    target = sig_y * rng.uniform(0.7, 1.1, size=(E, nip))
    S *= (target / nrm)[..., None, None]
    if two_d:
        S[..., 0, 2] = S[..., 2, 0] = S[..., 1, 2] = S[..., 2, 1] = 0.0
    Eps = _sym(rng, (E, nip), 2e-2, two_d)
    EpsPlas = _sym(rng, (E, nip), 1e-2, two_d)
    p = rng.normal(scale=1e8, size=(E, nip))
    if getattr(m, "groups", None):
        S, Eps, EpsPlas = S[:, 0], Eps[:, 0], EpsPlas[:, 0]
        p, evp = p[:, 0], evp[:, 0]
    return dict(coords=coords, du=du, v=v, a=a, disp=disp, S=S, Eps=Eps, EpsPlas=EpsPlas, p=p,
                evp=evp, dt=dt)
