"""Dense float64 PyTorch restatement of the soft-coverage model.

TEST INFRASTRUCTURE ONLY (a parity reference for the CUDA soft forward and adjoint).
Every pixel is evaluated against every triangle (no binning), in float64, and
torch autograd gives the reference gradients.  The model is the one of
``oracle/raster_ref.c`` (``orc_render_soft``): vertex transform of
``shaders/basic.vert:29-53`` with ``R = Rz(H) Ry(P) Rx(R)``
(``renderer/shader_context.py:47-84``), GL viewport into the scene's own
image, back faces culled, triangles not fully in front of the near plane
dropped, coverage ``D = prod_k sigmoid(e_k/sigma) T(d)`` with the C2 taper of the
distance ``d`` from the pixel to the triangle, the triangle's plane depth at the
pixel saturating smoothly beyond the triangle's farthest vertex depth (and
beyond the plane's vanishing line),
normalised linear depth, shading of ``shaders/basic.frag:33-38`` (unclamped),
softmax depth blend and alpha composite over the background.

Scene format: ``PBRRenderer.export_scene()`` (see ``oracle/oracle.py``).
Parameters are float64 tensors per node: ``pos [B,3]``, ``hpr [B,3]``,
``scale [B]``, ``color [B,4]``; plus ``light_dir [3]``.
"""
from __future__ import annotations

import numpy as np
import torch

CUT = 16.0
TAPER = 4.0
DEPTH_SAT = 0.125  # saturation depth of the extended plane, in units of zfar - znear


def params_from_nodes(nodes: list, requires_grad: bool = True) -> list[dict]:
    out = []
    for nd in nodes:
        if int(nd["mode"]) != 0:
            raise ValueError("the soft reference handles HPR-mode nodes only")
        d = {}
        for key, src in (("pos", "pos"), ("hpr", "rot"), ("scale", "scale"), ("color", "color")):
            d[key] = torch.tensor(np.asarray(nd[src], np.float64), dtype=torch.float64, requires_grad=requires_grad)
        out.append(d)
    return out


def rotation(hpr: torch.Tensor) -> torch.Tensor:
    h, p, r = hpr[:, 0], hpr[:, 1], hpr[:, 2]
    ch, sh, cp, sp, cr, sr = torch.cos(h), torch.sin(h), torch.cos(p), torch.sin(p), torch.cos(r), torch.sin(r)
    z, o = torch.zeros_like(h), torch.ones_like(h)
    Rz = torch.stack([ch, -sh, z, sh, ch, z, z, z, o], 1).reshape(-1, 3, 3)
    Ry = torch.stack([cp, z, sp, z, o, z, -sp, z, cp], 1).reshape(-1, 3, 3)
    Rx = torch.stack([o, z, z, z, cr, -sr, z, sr, cr], 1).reshape(-1, 3, 3)
    return Rz @ Ry @ Rx


def _taper(d: torch.Tensor, sigma: float) -> torch.Tensor:
    x = torch.clamp((CUT * sigma - d) / (TAPER * sigma), 0.0, 1.0)
    return x * x * x * (x * (x * 6 - 15) + 10)


def _seg_dist(px, py, ax, ay, bx, by):
    ux, uy = bx - ax, by - ay
    wx, wy = px - ax, py - ay
    l2 = ux * ux + uy * uy
    t = torch.clamp((wx * ux + wy * uy) / l2, 0.0, 1.0)
    dx, dy = px - (ax + t * ux), py - (ay + t * uy)
    return torch.sqrt(dx * dx + dy * dy + 1e-300)


def render(scene: dict, meshes: list, nodes: list, params: list[dict], light_dir: torch.Tensor) -> torch.Tensor:
    N, W, H = int(scene["N"]), int(scene["W"]), int(scene["H"])
    f64 = torch.float64
    VP = torch.tensor(np.asarray(scene["vp"], np.float32).reshape(N, 4, 4), dtype=f64)
    sigma, gamma = float(np.float32(scene["sigma"])), float(np.float32(scene["gamma"]))
    zn, zf = float(np.float32(scene["znear"])), float(np.float32(scene["zfar"]))
    amb = torch.tensor(np.asarray(scene["ambient"], np.float32), dtype=f64)
    lcol = torch.tensor(np.asarray(scene["lcol"], np.float32), dtype=f64)
    s = min(max(float(np.float32(scene["strength"])), 0.0), 1.0)
    bg = torch.tensor(np.asarray(scene["bg"], np.float32)[:3], dtype=f64)
    Ln = light_dir / torch.linalg.norm(light_dir)
    ys, xs = torch.meshgrid(torch.arange(H, dtype=f64) + 0.5, torch.arange(W, dtype=f64) + 0.5, indexing="ij")
    px, py = xs.reshape(-1), ys.reshape(-1)
    mesh_t = [(torch.tensor(np.asarray(m.positions, np.float32), dtype=f64),
               torch.tensor(np.asarray(m.normals, np.float32), dtype=f64),
               torch.tensor(np.asarray(m.indices), dtype=torch.long)) for m in meshes]
    frames = []
    for k in range(N):
        clips, norms, cols, smooth = [], [], [], []
        for nd, prm in zip(nodes, params):
            I, shared = int(nd["I"]), bool(nd["shared"])
            cnt = I if nd.get("counts") is None else min(int(nd["counts"][k]), I)
            if cnt == 0:
                continue
            ids = torch.arange(cnt) if shared else k * I + torch.arange(cnt)
            R = rotation(prm["hpr"][ids]) * prm["scale"][ids].reshape(-1, 1, 1)
            t = prm["pos"][ids]
            P, Nn, F = mesh_t[int(nd["mesh"])]
            world = torch.einsum("bij,vj->bvi", R, P) + t[:, None, :]
            clip = torch.einsum("ij,bvj->bvi", VP[k, :, :3], world) + VP[k, :, 3]
            nw = torch.einsum("bij,vj->bvi", R, Nn)
            nw = nw / torch.linalg.norm(nw, dim=-1, keepdim=True)
            clips.append(clip[:, F].reshape(-1, 3, 4))
            norms.append(nw[:, F].reshape(-1, 3, 3))
            cols.append(prm["color"][ids][:, None, :].expand(-1, F.shape[0], -1).reshape(-1, 4))
            is_smooth = bool(np.any(np.abs(np.asarray(meshes[int(nd["mesh"])].normals)[np.asarray(F)]
                                           - np.asarray(meshes[int(nd["mesh"])].normals)[np.asarray(F)][:, :1]) > 1e-7))
            smooth.append(torch.full((clip.shape[0] * F.shape[0],), is_smooth))
        if not clips:
            frames.append(bg[:, None].expand(3, H * W).reshape(3, H, W))
            continue
        c = torch.cat(clips)
        n = torch.cat(norms)
        col = torch.cat(cols)
        sm = torch.cat(smooth)
        iw = 1.0 / c[..., 3]
        sx = (c[..., 0] * iw + 1) * 0.5 * W
        sy = (1 - c[..., 1] * iw) * 0.5 * H
        area_pre = (sx[:, 1] - sx[:, 0]) * (sy[:, 2] - sy[:, 0]) - (sx[:, 2] - sx[:, 0]) * (sy[:, 1] - sy[:, 0])
        keep = (area_pre < 0) & ((c[..., 2] + c[..., 3]) >= 0).all(dim=1)
        keep = keep.detach()
        sel = torch.nonzero(keep).reshape(-1)
        if sel.numel() == 0:
            frames.append(bg[:, None].expand(3, H * W).reshape(3, H, W))
            continue
        order = torch.tensor([0, 2, 1])  # front faces: swap vertices 1 and 2
        sx, sy, iw = sx[sel][:, order], sy[sel][:, order], iw[sel][:, order]
        n, col, sm = n[sel][:, order], col[sel], sm[sel]
        area2 = (sx[:, 1] - sx[:, 0]) * (sy[:, 2] - sy[:, 0]) - (sx[:, 2] - sx[:, 0]) * (sy[:, 1] - sy[:, 0])
        E, e, fk, dseg = [], [], [], []
        for kk in range(3):
            a, b = (kk + 1) % 3, (kk + 2) % 3
            A_ = (sy[:, a] - sy[:, b])[:, None]
            B_ = (sx[:, b] - sx[:, a])[:, None]
            Ek = A_ * (px[None] - sx[:, a, None]) + B_ * (py[None] - sy[:, a, None])
            Lk = torch.sqrt(A_ * A_ + B_ * B_)
            ek = Ek / Lk
            E.append(Ek)
            e.append(ek)
            fk.append(torch.sigmoid(ek / sigma))
            dseg.append(_seg_dist(px[None], py[None], sx[:, a, None], sy[:, a, None], sx[:, b, None], sy[:, b, None]))
        emin0 = torch.minimum(torch.minimum(e[0], e[1]), e[2])
        dout = torch.where(emin0 < 0, torch.minimum(torch.minimum(dseg[0], dseg[1]), dseg[2]), torch.zeros_like(emin0))
        D = fk[0] * fk[1] * fk[2] * _taper(dout, sigma)
        Q = E[0] * iw[:, 0, None] + E[1] * iw[:, 1, None] + E[2] * iw[:, 2, None]
        qpos = (Q > 0).detach()
        Qs = torch.where(qpos, Q, torch.ones_like(Q))
        wv = 1.0 / iw  # vertex clip w [T,3]
        whi = torch.maximum(torch.maximum(wv[:, 0], wv[:, 1]), wv[:, 2])[:, None].expand_as(Q)
        sat = DEPTH_SAT * (zf - zn)
        w_raw = area2[:, None] / Qs
        beyond = (w_raw > whi).detach()
        w_sat = whi + sat * (1 - torch.exp(-torch.where(beyond, w_raw - whi, torch.zeros_like(w_raw)) / sat))
        w = torch.where(~qpos, whi + sat, torch.where(beyond, w_sat, w_raw))
        zs = (zf - w) / (zf - zn)
        emin = torch.minimum(torch.minimum(e[0], e[1]), e[2])
        valid = ((emin > -CUT * sigma) & (D > 0)).detach()
        # shading
        orient = torch.where(Q < 0, -1.0, 1.0).detach()[..., None]
        u_s = ((E[0] * iw[:, 0, None])[..., None] * n[:, None, 0] + (E[1] * iw[:, 1, None])[..., None] * n[:, None, 1]
               + (E[2] * iw[:, 2, None])[..., None] * n[:, None, 2]) * orient
        u_f = n[:, None, 0].expand_as(u_s)
        u = torch.where(sm[:, None, None], u_s, u_f)
        ulen = torch.linalg.norm(torch.where(valid[..., None], u, torch.ones_like(u)), dim=-1)
        ndl = torch.clamp((u * Ln).sum(-1) / ulen, min=0.0)
        light = amb[None, None, :] + ndl[..., None] * lcol[None, None, :]
        l = (1 - s) + light * s
        C = col[:, None, :3] * l
        Dm = torch.where(valid, D, torch.zeros_like(D))
        zsm = torch.where(valid, zs, torch.full_like(zs, -1e30))
        m = zsm.max(dim=0).values.detach()
        wts = Dm * torch.exp((torch.where(valid, zs, m[None].expand_as(zs)) - m[None]) / gamma)
        wts = torch.where(valid, wts, torch.zeros_like(wts))
        S = wts.sum(0)
        Cfg = (wts[..., None] * C).sum(0) / torch.where(S > 0, S, torch.ones_like(S))[:, None]
        Pn = torch.prod(1 - Dm, dim=0)
        A = 1 - Pn
        img = A[:, None] * Cfg + (1 - A)[:, None] * bg[None]
        frames.append(img.T.reshape(3, H, W))
    return torch.stack(frames)
