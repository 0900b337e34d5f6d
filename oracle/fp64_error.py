"""Error of float32 results against the FP64 twin, with bounds derived from
float32 rounding (test infrastructure only).

u = 2^-24 is the unit roundoff of float32.  With the float32 grid
description (origin o, spacing s, extent minimum m), the FP64 twin computes a
point coordinate as c = o + s (i + m) in double (exact to 2^-53), the float32
path as fl(o + fl(s (i + m))), which is off by at most
    E = u (|s (i + m)| + |c|) (1 + u)                                    (1)

Marching cubes (dax/worklet/MarchingCubes.h:160-161, dax/math/VectorAnalysis.h:60-63):
* weight w = (iso - fA) / (fB - fA): two rounded subtractions and a rounded
  division of exactly widened float32 values, so
    |w32 - w64| <= ((1 + u)^2 / (1 - u) - 1) |w64| < 3.01 u |w64|         (2)
* position along the edge's axis p = cA + w (cB - cA): the twin uses the
  exact spacing for cB - cA; the float32 path has (1) at both ends, the
  rounded difference, product and sum, and (2), so
    |p32 - p64| <= 3 E + 5 u |s| + u |p|                                (3)
  and the two other components are cA itself, off by E.
CellGradient (dax/exec/Derivative.h:37-75): the eight products f_v * (+-0.25)
are exact; seven rounded additions give an error of at most 7u sum|0.25 f_v|
(plus second-order terms); the width x6 - x0 is off from s by at most
2E + u|s| (relative rho), and the quotient is rounded once, so
    |g32 - g64| <= 8 u A / |w| + (rho + 2u) |g64|,  A = sum_v 0.25 |f_v|   (4)
"""
import numpy as np

U = 2.0 ** -24


def _axis_terms(origin, spacing, emin, dims):
    """Per axis: max coordinate error E (1), max |coordinate|, |spacing|."""
    out = []
    for a in range(3):
        i = np.arange(dims[a], dtype=np.float64) + emin[a]
        s = float(np.float32(spacing[a]))
        o = float(np.float32(origin[a]))
        c = o + s * i
        E = U * (np.abs(s * i) + np.abs(c)).max() * (1 + U)
        out.append((E, float(np.abs(c).max()), abs(s)))
    return out


def position_bound(origin, spacing, emin, dims):
    """(3) in units of each axis' spacing: the largest over the axes."""
    b = 0.0
    for E, C, s in _axis_terms(origin, spacing, emin, dims):
        if s > 0:
            b = max(b, (3 * E + 5 * U * s + U * C) / s)
    return b


def mc_error_stats(verts32, w32, r64, origin, spacing, emin, dims):
    """Position error in units of the spacing (per component, per axis'
    spacing) and weight error of the float32 surface against the twin's;
    `r64` from oracle.Fp64Twin.mc_generate on the same inputs."""
    s = np.abs(np.asarray([float(np.float32(x)) for x in spacing]))
    v32 = np.asarray(verts32, np.float64)
    pe = np.abs(v32 - r64["verts"]) / s[None, :]
    we = np.abs(np.asarray(w32, np.float64) - r64["rec_w"])
    wb = 3.01 * U * np.abs(r64["rec_w"]) + 2.0 ** -149
    flat = pe.ravel()
    return {
        "vertices": int(v32.shape[0]),
        "pos_err_max_spacings": float(flat.max()) if flat.size else 0.0,
        "pos_err_p50_spacings": float(np.percentile(flat, 50)) if flat.size else 0.0,
        "pos_err_p99_spacings": float(np.percentile(flat, 99)) if flat.size else 0.0,
        "pos_err_p999_spacings": float(np.percentile(flat, 99.9)) if flat.size else 0.0,
        "pos_bound_spacings": position_bound(origin, spacing, emin, dims),
        "weight_err_max": float(we.max()) if we.size else 0.0,
        "weight_err_over_bound_max": float((we / wb).max()) if we.size else 0.0,
    }


def gradient_error_stats(g32, g64, field, origin, spacing, emin, dims, planes=64):
    """CellGradient error against the twin: the largest ratio of the error
    to bound (4), the largest error relative to A / |w| (the scale of the
    eight terms), and the largest relative error over cells whose gradient
    component is at least 1e-3 of the largest; z-chunks of `planes` cell
    planes keep the temporaries small."""
    nx, ny, nz = dims
    f3 = np.asarray(field, np.float32).reshape(nz, ny, nx)
    g32 = np.asarray(g32).reshape(nz - 1, ny - 1, nx - 1, 3)
    g64 = np.asarray(g64).reshape(nz - 1, ny - 1, nx - 1, 3)
    terms = _axis_terms(origin, spacing, emin, dims)
    rho = [(2 * E + U * s) / s for (E, C, s) in terms]
    gmax = np.abs(g64).max(axis=(0, 1, 2))
    over, norm, rel = 0.0, 0.0, 0.0
    for k0 in range(0, nz - 1, planes):
        k1 = min(nz - 1, k0 + planes)
        f = np.abs(f3[k0:k1 + 1].astype(np.float64))
        A = 0.25 * (f[:-1, :-1, :-1] + f[:-1, :-1, 1:] + f[:-1, 1:, :-1] + f[:-1, 1:, 1:] +
                    f[1:, :-1, :-1] + f[1:, :-1, 1:] + f[1:, 1:, :-1] + f[1:, 1:, 1:])
        for a in range(3):
            s = terms[a][2]
            e = np.abs(g32[k0:k1, ..., a].astype(np.float64) - g64[k0:k1, ..., a])
            ref = np.abs(g64[k0:k1, ..., a])
            bound = 8 * U * A / s + (rho[a] + 2 * U) * ref
            over = max(over, float((e / np.maximum(bound, 1e-300)).max()))
            norm = max(norm, float((e / np.maximum(A / s, 1e-300)).max()))
            big = ref >= 1e-3 * gmax[a]
            if big.any():
                rel = max(rel, float((e[big] / ref[big]).max()))
    return {"cells": int((nx - 1) * (ny - 1) * (nz - 1)),
            "err_over_bound_max": over,
            "err_over_term_scale_max": norm,
            "rel_err_max_where_above_1e-3_of_max": rel,
            "width_rel_err_bound": max(rho)}
