"""CPU ORACLE — test infrastructure only (the product never imports this file).

The differentiable rollout restated in torch float64 on the CPU, element colour by element colour,
so that torch's autograd — not a hand derivation — provides its gradient.  Tests compare the
oracle's hand-written FP64 adjoint (ORC_DiffBackward, oracle/diff_oracle.inc) and, through it,
the CUDA adjoint with this gradient.  Topology and constants come from an oracle session
(ORC_ExportTopology), so both sides solve the same mesh.

Forward expressions follow the plain substep of the reference (V/xpbd/xpbd_solver.cu, "V/" =
endoscopic_tissue/native/vendor/cuda/): predict 393-412, lattice edges 484-524, unguarded
Neo-Hookean tets 749-829, capsule contact 1049-1093 (shaft only, no jaw), velocity 871-919;
per-tet compliance over h^2 = h^-2 / (baked stiffness / (exp(theta) E0)).
"""
from __future__ import annotations

import ctypes as ct

import numpy as np
import torch

P = ct.c_void_p


def _p(a):
    return a.ctypes.data_as(P)


def export_topology(dll) -> dict:
    sizes = np.zeros(5, dtype=np.int32)
    assert dll.ORC_TopologySizes(_p(sizes)) == 0
    N, E, T, nec, ntc = (int(x) for x in sizes)
    t = dict(N=N, E=E, T=T, eIJ=np.zeros((E, 2), np.int32), eRest=np.zeros(E), eLive=np.zeros(E, np.int32),
             eColOff=np.zeros(nec + 1, np.int32), tIds=np.zeros((T, 4), np.int32), tType=np.zeros(T, np.int32),
             tLive=np.zeros(T, np.int32), tOrder=np.zeros(T, np.int32), tColOff=np.zeros(ntc + 1, np.int32),
             typeB=np.zeros((6, 3, 3)), tStiff=np.zeros((T, 2)), invMass=np.zeros(N), ext=np.zeros((N, 3)))
    rc = dll.ORC_ExportTopology(*(_p(t[k]) for k in ("eIJ", "eRest", "eLive", "eColOff", "tIds", "tType", "tLive", "tOrder", "tColOff",
                                                       "typeB", "tStiff", "invMass", "ext")))
    assert rc == 0
    params = np.zeros(10)
    assert dll.ORC_Parameters(_p(params)) == 0
    for k, v in zip(("ks", "betaS", "omega", "strainDamping", "damping", "alpha", "contactAlpha", "ccdVelThresh", "ccdMaxDisp",
                     "ccdOmega"), params):
        t[k] = float(v)
    return t


def _cross(a, b):
    return torch.linalg.cross(a, b, dim=-1)


def _safe(x, ok):
    """x where ok, else 1 (keeps masked-out branches finite so their zero gradient stays zero)."""
    return torch.where(ok, x, torch.ones_like(x))


def rollout(topo: dict, origin_pos, origin_vel, theta: torch.Tensor, path: torch.Tensor | None, radius: float, dt: float, substeps: int,
            frames: int, young: float) -> torch.Tensor:
    """Final node positions [N, 3] (float64, differentiable in theta and path)."""
    f64 = dict(dtype=torch.float64)
    h = float(np.float32(dt)) / substeps
    invH2 = 1.0 / (h * h)
    alpha_tilde = 1.0 / (topo["ks"] * h * h)
    gamma = alpha_tilde * topo["betaS"] * h
    omega = topo["omega"]
    doh = max(0.0, topo["strainDamping"]) / h
    scale = 1.0 + doh
    vel_scale = (1.0 - topo["damping"]) / (1.0 + topo["alpha"] * h)
    contact_alpha = topo["contactAlpha"] / (h * h)
    w = torch.tensor(topo["invMass"], **f64)
    movable = (w > 0)[:, None]
    ext = torch.tensor(topo["ext"], **f64)
    stiff = torch.tensor(topo["tStiff"], **f64)
    s = 1.0 / (torch.exp(theta) * young)
    aD, aH = invH2 / (stiff[:, 0] * s), invH2 / (stiff[:, 1] * s)
    typeB = torch.tensor(topo["typeB"], **f64)
    eIJ = torch.tensor(topo["eIJ"], dtype=torch.long)
    eRest = torch.as_tensor(topo["eRest"], **f64)
    edge_sets = []
    for c in range(len(topo["eColOff"]) - 1):
        e = np.arange(topo["eColOff"][c], topo["eColOff"][c + 1])
        e = e[topo["eLive"][e] != 0]
        edge_sets.append(torch.tensor(e, dtype=torch.long))
    tet_sets = []
    for c in range(len(topo["tColOff"]) - 1):
        t = topo["tOrder"][topo["tColOff"][c]:topo["tColOff"][c + 1]]
        t = t[topo["tLive"][t] != 0]
        tet_sets.append(torch.tensor(t, dtype=torch.long))
    tIds = torch.tensor(topo["tIds"], dtype=torch.long)
    tType = torch.tensor(topo["tType"], dtype=torch.long)
    x = torch.as_tensor(origin_pos, **f64).clone()
    v = torch.as_tensor(origin_vel, **f64).clone()
    for f in range(frames):
        for sub in range(substeps):
            tl = min(1.0, (sub + 1) / substeps)
            q = x
            v = torch.where(movable, v + (ext * w[:, None]) * h, v)
            x = torch.where(movable, x + v * h, x)
            for e in edge_sets:
                i, j = eIJ[e, 0], eIJ[e, 1]
                pi, pj, wi, wj = x[i], x[j], w[i], w[j]
                d = pi - pj
                L = d.norm(dim=-1)
                ok = ((wi + wj) > 0) & (L >= 1e-9)
                Ls = _safe(L, ok)
                n = d / Ls[:, None]
                C = Ls - eRest[e]
                gdx = (n * ((pi - q[i]) - (pj - q[j]))).sum(-1)
                dl = (-C - gamma * gdx) / ((1 + gamma) * (wi + wj) + alpha_tilde)
                ap = omega * dl
                ni = torch.where(ok[:, None], pi + n * (wi * ap)[:, None], pi)
                nj = torch.where(ok[:, None], pj - n * (wj * ap)[:, None], pj)
                x = x.index_put((i,), ni).index_put((j,), nj)
            for t in tet_sets:
                ids = tIds[t]
                p, qq, ww = x[ids], q[ids], w[ids]
                Bm = typeB[tType[t]]
                e = p[:, 1:] - p[:, :1]                                   # e[:, k] = p_{k+1} - p_0
                F = torch.einsum("tki,tkc->tci", e, Bm)                    # F[:, c] = column c
                I1 = (F * F).sum((1, 2))
                cof = torch.stack((_cross(F[:, 1], F[:, 2]), _cross(F[:, 2], F[:, 0]), _cross(F[:, 0], F[:, 1])), 1)
                J = (F[:, 0] * cof[:, 0]).sum(-1)
                pJ = torch.clamp(J, min=0.05)
                iso = pJ ** (-2.0 / 3.0)
                q0 = torch.clamp(iso * I1 - 3.0, min=0.0)
                CD = torch.sqrt(torch.clamp(q0, min=1e-12))
                dev = 1.0 / CD
                vol = torch.where(J > 0.05, iso * I1 / (3.0 * pJ), torch.zeros_like(J))
                CH = J - 1.0
                gh = torch.einsum("tcj,tji->tci", Bm, cof)                # gh_{c+1} = sum_j Bm[c][j] cof_j
                G = torch.einsum("tcj,tji->tci", Bm, F)
                gd = (G * iso[:, None, None] - gh * vol[:, None, None]) * dev[:, None, None]
                gd = torch.cat((-gd.sum(1, keepdim=True), gd), 1)
                gh = torch.cat((-gh.sum(1, keepdim=True), gh), 1)
                dx = p - qq
                dd = (ww * (gd * gd).sum(-1)).sum(-1)
                dh = (ww * (gd * gh).sum(-1)).sum(-1)
                vd = (gd * dx).sum((1, 2))
                vh = (gh * dx).sum((1, 2))
                eAd, eAh = aD[t] / scale, aH[t] / scale
                A = dd + eAd
                As = _safe(A, A > 0)
                gam = dh / As
                r = gh - gd * gam[:, None, None]
                schur = eAh + eAd * gam * gam + (ww * (r * r).sum(-1)).sum(-1)
                ok = (A > 0) & (schur > 0)
                ss = _safe(schur, ok)
                rd = (-CD - doh * vd) / scale
                rh = (-CH - (scale - 1.0) * vh) / scale
                dlH = omega * (rh - gam * rd) / ss
                dlD = (omega * rd - dh * dlH) / As
                o = p + (gd * dlD[:, None, None] + gh * dlH[:, None, None]) * ww[:, :, None]
                new = torch.where(ok[:, None, None], o, p)
                x = x.index_put((ids.reshape(-1),), new.reshape(-1, 3))
            if path is not None:
                sa = path[f, :3] * (1 - tl) + path[f + 1, :3] * tl
                sb = path[f, 3:] * (1 - tl) + path[f + 1, 3:] * tl
                ab = sb - sa
                ab2 = (ab * ab).sum()
                raw = ((x - sa) * ab).sum(-1) / ab2 if float(ab2) > 1e-12 else torch.zeros(len(x), **f64)
                tt = torch.clamp(raw, 0.0, 1.0)
                dv = x - (sa + ab * tt[:, None])
                dist = dv.norm(dim=-1)
                C = dist - radius
                nrm = dist > 1e-9
                n = torch.where(nrm[:, None], dv / _safe(dist, nrm)[:, None], torch.tensor((0.0, 1.0, 0.0), **f64).expand_as(dv))
                gate = (w > 0) & (C < 0) & (-(v * n).sum(-1) > topo["ccdVelThresh"])
                ap = topo["ccdOmega"] * (-C / (w + contact_alpha))
                corr = n * (w * ap)[:, None]
                cl = corr.norm(dim=-1)
                cap = cl > topo["ccdMaxDisp"]
                corr = torch.where(cap[:, None], corr * (topo["ccdMaxDisp"] / _safe(cl, cap))[:, None], corr)
                x = torch.where(gate[:, None], x + corr, x)
            v = torch.where(movable, (x - q) * (1.0 / h) * vel_scale, torch.zeros_like(x))
    return x
