"""ORACLE (test infrastructure only): LDR-FLIP of the reference's evaluation.

Restates scripts/flip_loss.py (LDRFLIPLoss.forward, compute_ldrflip,
generate_spatial_filter, spatial_filter, feature_detection, hunt_adjustment,
hyab, redistribute_errors, color_space_transform; the published LDR-FLIP of
Andersson et al., HPG 2020) in float64 numpy, with the 2-D filters applied as
the reference does (direct correlation with replicate padding).  Pinned
against the reference's own code run with torch on the CPU
(tests/golden/metrics/flip.npz, written by tests/golden/make_golden.py flip).
"""
from __future__ import annotations

import math

import numpy as np

QC, QF, PC, PT, EPS = 0.7, 0.5, 0.4, 0.95, 1e-15
DEFAULT_PPD = (0.7 * 3840 / 0.7) * math.pi / 180  # eval.py's default viewing condition

_ILLUM = np.array([0.950428545, 1.000000000, 1.088900371])
_INV_ILLUM = np.array([1.052156925, 1.000000000, 0.918357670])
_LIN2XYZ = np.array([[10135552 / 24577794, 8788810 / 24577794, 4435075 / 24577794],
                     [2613072 / 12288897, 8788810 / 12288897, 887015 / 12288897],
                     [1425312 / 73733382, 8788810 / 73733382, 70074185 / 73733382]])
_XYZ2LIN = np.array([[3.241003275, -1.537398934, -0.498615861],
                     [-0.969224334, 1.875930071, 0.041554224],
                     [0.055639423, -0.204011202, 1.057148933]])


def srgb_to_ycxcz(rgb: np.ndarray) -> np.ndarray:
    """(3, H, W) sRGB in [0, 1] -> YCxCz (flip_loss.py color_space_transform 'srgb2ycxcz')."""
    lim = 0.04045
    lin = np.where(rgb > lim, ((np.maximum(rgb, lim) + 0.055) / 1.055) ** 2.4, rgb / 12.92)
    xyz = np.einsum("ij,jhw->ihw", _LIN2XYZ, lin) * _INV_ILLUM[:, None, None]
    return np.stack([116 * xyz[1] - 16, 500 * (xyz[0] - xyz[1]), 200 * (xyz[1] - xyz[2])])


def ycxcz_to_linrgb(c: np.ndarray) -> np.ndarray:
    y = (c[0] + 16) / 116
    x, z = y + c[1] / 500, y - c[2] / 200
    xyz = np.stack([x, y, z]) * _ILLUM[:, None, None]
    return np.einsum("ij,jhw->ihw", _XYZ2LIN, xyz)


def linrgb_to_lab(rgb: np.ndarray) -> np.ndarray:
    xyz = np.einsum("ij,jhw->ihw", _LIN2XYZ, rgb) * _INV_ILLUM[:, None, None]
    d = 6 / 29
    f = np.where(xyz > d ** 3, np.maximum(xyz, d ** 3) ** (1 / 3), xyz / (3 * d * d) + 4 / 29)
    return np.stack([116 * f[1] - 16, 500 * (f[0] - f[1]), 200 * (f[1] - f[2])])


def hunt(lab: np.ndarray) -> np.ndarray:
    return np.stack([lab[0], 0.01 * lab[0] * lab[1], 0.01 * lab[0] * lab[2]])


def hyab(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    d = a - b
    return np.sqrt(np.maximum(d[0] ** 2, EPS)) + np.sqrt(d[1] ** 2 + d[2] ** 2)


def csf_kernel(ppd: float, channel: str):
    """generate_spatial_filter: (2r+1)^2 normalised kernel and r."""
    p = {"A": (1, 0.0047, 0, 1e-5), "RG": (1, 0.0053, 0, 1e-5), "BY": (34.1, 0.04, 13.5, 0.025)}[channel]
    a1, b1, a2, b2 = p
    r = int(math.ceil(3 * math.sqrt(0.04 / (2 * math.pi ** 2)) * ppd))
    dx = 1.0 / ppd
    x, y = np.meshgrid(range(-r, r + 1), range(-r, r + 1))
    z = (x * dx) ** 2 + (y * dx) ** 2
    g = a1 * math.sqrt(math.pi / b1) * np.exp(-math.pi ** 2 * z / b1) + a2 * math.sqrt(math.pi / b2) * np.exp(-math.pi ** 2 * z / b2)
    return g / g.sum(), r


def feature_kernel(ppd: float, kind: str):
    """feature_detection's x-direction kernel (edge: first derivative, point: second)."""
    sd = 0.5 * 0.082 * ppd
    r = int(math.ceil(3 * sd))
    x, y = np.meshgrid(range(-r, r + 1), range(-r, r + 1))
    g = np.exp(-(x ** 2 + y ** 2) / (2 * sd * sd))
    gx = -x * g if kind == "edge" else (x ** 2 / (sd * sd) - 1) * g
    neg, pos = -gx[gx < 0].sum(), gx[gx > 0].sum()
    return np.where(gx < 0, gx / neg, gx / pos), r


def correlate_replicate(img: np.ndarray, k: np.ndarray, r: int) -> np.ndarray:
    """conv2d (a correlation) of (H, W) with a (2r+1)^2 kernel after replicate padding."""
    h, w = img.shape
    p = np.pad(img, r, mode="edge")
    out = np.zeros((h, w))
    for dy in range(2 * r + 1):
        for dx in range(2 * r + 1):
            if k[dy, dx] != 0.0:
                out += k[dy, dx] * p[dy:dy + h, dx:dx + w]
    return out


def cmax() -> float:
    green = hunt(linrgb_to_lab(np.array([0.0, 1.0, 0.0]).reshape(3, 1, 1)))
    blue = hunt(linrgb_to_lab(np.array([0.0, 0.0, 1.0]).reshape(3, 1, 1)))
    return float(hyab(green, blue)[0, 0] ** QC)


def flip_map(test: np.ndarray, reference: np.ndarray, ppd: float = DEFAULT_PPD) -> np.ndarray:
    """Per-pixel LDR-FLIP of two (H, W, 3|4) uint8 images (RGB / 255, alpha dropped)."""
    t = np.moveaxis(np.asarray(test)[..., :3].astype(np.float64) / 255.0, -1, 0)
    r = np.moveaxis(np.asarray(reference)[..., :3].astype(np.float64) / 255.0, -1, 0)
    t_opp, r_opp = srgb_to_ycxcz(np.clip(t, 0, 1)), srgb_to_ycxcz(np.clip(r, 0, 1))
    kernels = [csf_kernel(ppd, c) for c in ("A", "RG", "BY")]
    rad = max(k[1] for k in kernels)

    def color(opp):
        filt = np.stack([correlate_replicate(opp[c], kernels[c][0], rad) for c in range(3)])
        return hunt(linrgb_to_lab(np.clip(ycxcz_to_linrgb(filt), 0.0, 1.0)))

    power = hyab(color(r_opp), color(t_opp)) ** QC
    cm = cmax()
    pccmax = PC * cm
    de_c = np.where(power < pccmax, (PT / pccmax) * power, PT + ((power - pccmax) / (cm - pccmax)) * (1.0 - PT))

    ke, re = feature_kernel(ppd, "edge")
    kp, rp = feature_kernel(ppd, "point")

    def features(opp):
        y = (opp[0] + 16) / 116
        ex, ey = correlate_replicate(y, ke, re), correlate_replicate(y, ke.T, re)
        px, py = correlate_replicate(y, kp, rp), correlate_replicate(y, kp.T, rp)
        return np.hypot(ex, ey), np.hypot(px, py)

    er, pr = features(r_opp)
    et, pt = features(t_opp)
    de_f = np.maximum(np.abs(er - et), np.abs(pt - pr))
    de_f = np.maximum(de_f, EPS)
    de_f = ((1 / math.sqrt(2)) * de_f) ** QF
    return de_c ** (1 - de_f)


def flip(test: np.ndarray, reference: np.ndarray, ppd: float = DEFAULT_PPD) -> float:
    """Mean LDR-FLIP (eval.py's flip_fn(render, ground_truth))."""
    return float(flip_map(test, reference, ppd).mean())
