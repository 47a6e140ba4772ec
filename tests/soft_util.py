"""Helpers shared by the soft-mode tests: finite differences on the FP64
oracle (Richardson-extrapolated central differences) and relative errors."""
import numpy as np

from oracle import oracle

KEY_SRC = {"pos": "pos", "hpr": "rot", "scale": "scale", "color": "color"}


def loss_of(scene, meshes, nodes, target):
    img = oracle.render_soft(scene, meshes, nodes, out_dtype=np.float64)
    return float(((img - target) ** 2).mean())


def fd_param(scene, meshes, nodes, target, ni, key, idx, h=1e-4, richardson=True):
    """d loss / d nodes[ni][key].flat[idx] by central differences in FP64.
    The perturbed value is rounded to float32 (what the renderer reads) and
    the secant uses the exact rounded step."""
    def secant(step):
        vals = []
        xs = []
        for sgn in (1.0, -1.0):
            nn = [dict(n) for n in nodes]
            arr = np.array(nn[ni][KEY_SRC[key]], np.float32).copy()
            arr.reshape(-1)[idx] = np.float32(float(arr.reshape(-1)[idx]) + sgn * step)
            nn[ni][KEY_SRC[key]] = arr
            vals.append(loss_of(scene, meshes, nn, target))
            xs.append(float(arr.reshape(-1)[idx]))
        return (vals[0] - vals[1]) / (xs[0] - xs[1])
    d1 = secant(h)
    if not richardson:
        return d1
    d2 = secant(h / 2)
    return (4 * d2 - d1) / 3


def fd_light(scene, meshes, nodes, target, i, h=1e-4, richardson=True):
    def secant(step):
        vals, xs = [], []
        for sgn in (1.0, -1.0):
            d = list(np.asarray(scene["ldir"], np.float32))
            d[i] = np.float32(float(d[i]) + sgn * step)
            vals.append(loss_of(dict(scene, ldir=tuple(d)), meshes, nodes, target))
            xs.append(float(d[i]))
        return (vals[0] - vals[1]) / (xs[0] - xs[1])
    d1 = secant(h)
    if not richardson:
        return d1
    return (4 * secant(h / 2) - d1) / 3


def rel_err(got, want):
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    den = np.linalg.norm(want)
    return float(np.linalg.norm(got - want) / den) if den > 0 else float(np.linalg.norm(got))
