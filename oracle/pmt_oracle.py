"""CPU ORACLE of the detection step (test infrastructure only).

numpy restatement, in FP32 like the device, of photon hits -> PMT hits:
check_pmt_hit for a POM with POMAcceptance (src/pom.jl:246-305), for a
homogeneous module (src/detection.jl:57-84), for a DOM with its wavelength
acceptance (src/dom.jl:96-134), for a generic multi-PMT module
(src/detection.jl:90-131, the PMT drawn by StatsBase 0.34's weighted sample:
the first index whose running weight sum reaches U * sum, else the last), and
the quantum
efficiency of calc_pe_weight! (src/processing.jl:179-205), drawing u1, u2 from
the same Philox4x32-10 stream as photonpropagation.jl_gb300/csrc/pp_pmt.cu
(counter (row, 0x504d5400, 0), key = seed) so that every decision can be
replayed.  philox4x32_10 here is vectorised numpy, pinned against the C
oracle's Random123-checked Philox.
"""
from __future__ import annotations

import numpy as np

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF
PMT_STREAM = 0x504D5400


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Arrays of 32-bit counter words (any integer dtype) -> 4 uint32 arrays."""
    c = [np.asarray(v, np.uint64) & MASK for v in (c0, c1, c2, c3)]
    k0 = np.uint64(k0 & MASK)
    k1 = np.uint64(k1 & MASK)
    for r in range(10):
        if r:
            k0 = (k0 + np.uint64(W0)) & np.uint64(MASK)
            k1 = (k1 + np.uint64(W1)) & np.uint64(MASK)
        p0 = np.uint64(M0) * c[0]
        p1 = np.uint64(M1) * c[2]
        c = [((p1 >> np.uint64(32)) ^ c[1] ^ k0) & np.uint64(MASK), p1 & np.uint64(MASK),
             ((p0 >> np.uint64(32)) ^ c[3] ^ k1) & np.uint64(MASK), p0 & np.uint64(MASK)]
    return [v.astype(np.uint32) for v in c]


def u01(x):
    """24-bit uniform in (0, 1], as the device's u01."""
    return ((np.asarray(x, np.uint32) >> 8) + 1).astype(np.float32) * np.float32(2.0 ** -24)


def interp0(x, y, v):
    """Linear interpolation, 0 outside the knots, FP32 like the device."""
    x = np.asarray(x, np.float32)
    y = np.asarray(y, np.float32)
    v = np.asarray(v, np.float32)
    out = np.zeros(v.shape, np.float32)
    inside = (v >= x[0]) & (v <= x[-1])
    hi = np.clip(np.searchsorted(x, v, side="right"), 1, len(x) - 1)
    lo = hi - 1
    t = (v - x[lo]) / (x[hi] - x[lo])
    val = (t * (y[hi] - y[lo]) + y[lo]).astype(np.float32)
    out[inside] = val[inside]
    return out


def rayleigh_pdf(x, sigma):
    s2 = np.float32(sigma) * np.float32(sigma)
    return (x / s2 * np.exp(-x * x / (np.float32(2.0) * s2))).astype(np.float32)


def _dom(dirs, wl, u1, u2, m):
    """DOM: detected (as PMT 1) when u1 * polymax < poly(cos zenith) and, with
    the wavelength acceptance on, u2 < wl_acc(wavelength)."""
    z = np.asarray(m["zenith_axis"], np.float32)
    cz = (dirs.astype(np.float64) @ z.astype(np.float64)).astype(np.float32)
    poly = np.zeros(len(cz), np.float32)
    for c in np.asarray(m["poly"], np.float32)[::-1]:  # Horner, one rounding per step
        poly = (poly.astype(np.float64) * cz + np.float64(c)).astype(np.float32)
    ang = (u1 * np.float32(m["polymax"])).astype(np.float32) < poly
    wl_ok = u2 < interp0(m["wl"], m["wl_acc"], wl) if m.get("apply_wl", True) else True
    return np.where(ang & wl_ok, 1, 0).astype(np.int32)


def _multipmt(pos, dirs, wl, u1, u2, centre, radius, m):
    """Multi-PMT: hit when u1 <= sum_k max(dir . q_k, 0) * area / (pi r^2),
    then the PMT of a cumulative scan of w_k = -(rel . p_k) for u2."""
    qm = np.asarray(m["pmt_dir_module"], np.float32)
    qo = np.asarray(m["pmt_dir"], np.float32)
    n_pmt = len(qm)
    proj = np.zeros(len(wl), np.float32)
    for k in range(n_pmt):
        c = (dirs[:, 0] * qm[k, 0] + dirs[:, 1] * qm[k, 1] + dirs[:, 2] * qm[k, 2]).astype(
            np.float32)
        proj = np.where(c > 0, (proj + c).astype(np.float32), proj)
    prob = ((proj * np.float32(m["pmt_area"])).astype(np.float32) /
            ((np.float32(3.14159265358979) * radius).astype(np.float32) * radius)).astype(
        np.float32)
    hit = u1 <= prob
    rel = ((pos - centre) * (np.float32(1.0) / radius)).astype(np.float32)
    w = np.stack([-(rel[:, 0] * qo[k, 0] + rel[:, 1] * qo[k, 1] + rel[:, 2] * qo[k, 2])
                  for k in range(n_pmt)], axis=1).astype(np.float32)
    wsum = np.zeros(len(wl), np.float32)
    for k in range(n_pmt):
        wsum = (wsum + w[:, k]).astype(np.float32)
    target = (u2 * wsum).astype(np.float32)
    chosen = np.full(len(wl), n_pmt, np.int32)
    cw = np.zeros(len(wl), np.float32)
    done = np.zeros(len(wl), bool)
    for k in range(n_pmt):
        cw = (cw + w[:, k]).astype(np.float32)
        now = (~done) & ~(cw < target)
        chosen[now] = k + 1
        done |= now
    return np.where(hit, chosen, 0).astype(np.int32), interp0(m["qe_wavelength"], m["qe"], wl)


def detect(positions, wavelengths, module_index, targets, model, seed, directions=None):
    """PMT id per hit (0 = not detected) and the QE weight.

    targets: list of dicts {position, radius, kind ('pom'|'homogeneous'|'dom'|
    'multipmt'), active_area}; model: dict with acc_wavelength, acc_group1,
    acc_group2, sigma_group1, sigma_group2, qe_wavelength, qe, pmt_dir (16 x 3),
    pmt_group (16) for POMs, and sub-dicts model['dom'] (poly, polymax,
    zenith_axis, wl, wl_acc, apply_wl) and model['multipmt'] (pmt_dir_module,
    pmt_dir, pmt_area, qe_wavelength, qe) for those kinds; directions (n x 3)
    are needed by DOMs and multi-PMT modules."""
    pos = np.asarray(positions, np.float32).reshape(-1, 3)
    dirs = None if directions is None else np.asarray(directions, np.float32).reshape(-1, 3)
    wl = np.asarray(wavelengths, np.float32)
    mi = np.asarray(module_index, np.int64)
    n = len(wl)
    rows = np.arange(n, dtype=np.uint64)
    r = philox4x32_10(rows & MASK, rows >> np.uint64(32), np.full(n, PMT_STREAM), np.zeros(n),
                      seed & MASK, (seed >> 32) & MASK)
    u1, u2 = u01(r[0]), u01(r[1])
    ids = np.zeros(n, np.int32)
    qe = np.zeros(n, np.float32)
    for t_ix, t in enumerate(targets):
        sel = np.flatnonzero(mi == t_ix + 1)
        if not len(sel):
            continue
        radius = np.float32(t["radius"])
        if t["kind"] == "homogeneous":
            frac = np.float32(t["active_area"]) / (np.float32(4.0) * np.float32(3.14159265358979) *
                                                  radius * radius)
            ids[sel] = (u1[sel] < frac).astype(np.int32)
            qe[sel] = 1.0
            continue
        if t["kind"] == "dom":
            ids[sel] = _dom(dirs[sel], wl[sel], u1[sel], u2[sel], model["dom"])
            qe[sel] = 1.0
            continue
        if t["kind"] == "multipmt":
            ids[sel], qe[sel] = _multipmt(pos[sel], dirs[sel], wl[sel], u1[sel], u2[sel],
                                          np.asarray(t["position"], np.float32), radius,
                                          model["multipmt"])
            continue
        m = model
        c0 = np.asarray(t["position"], np.float32)
        inv_r = np.float32(1.0) / radius
        rel = (pos[sel] - c0) * inv_r
        acc1 = interp0(m["acc_wavelength"], m["acc_group1"], wl[sel])
        acc2 = interp0(m["acc_wavelength"], m["acc_group2"], wl[sel])
        dirs = np.asarray(m["pmt_dir"], np.float32)
        prob = np.zeros((len(sel), 16), np.float32)
        for k in range(16):
            c = rel[:, 0] * dirs[k, 0] + rel[:, 1] * dirs[k, 1] + rel[:, 2] * dirs[k, 2]
            pt = np.arccos(np.clip(c, -1, 1)).astype(np.float32)
            g1 = m["pmt_group"][k] == 1
            s = np.sin(pt).astype(np.float32)
            sig = m["sigma_group1"] if g1 else m["sigma_group2"]
            with np.errstate(divide="ignore", invalid="ignore"):
                w = np.where(s != 0, rayleigh_pdf(pt, sig) / (np.float32(0.5) * s), 0.0)
            prob[:, k] = (w.astype(np.float32) * (acc1 if g1 else acc2) *
                          np.float32(0.125)).astype(np.float32)
        total = np.zeros(len(sel), np.float32)
        for k in range(16):
            total = (total + prob[:, k]).astype(np.float32)
        hit = u1[sel] < total
        target = (u2[sel] * total).astype(np.float32)
        cum = np.zeros(len(sel), np.float32)
        chosen = np.full(len(sel), 16, np.int32)
        done = np.zeros(len(sel), bool)
        for k in range(16):
            cum = (cum + prob[:, k]).astype(np.float32)
            now = (~done) & (cum >= target)
            chosen[now] = k + 1
            done |= now
        ids[sel] = np.where(hit, chosen, 0)
        qe[sel] = interp0(m["qe_wavelength"], m["qe"], wl[sel])
    return ids, qe


def detection_probability(positions, wavelengths, target, model):
    """FP64 probability that a photon at each position is detected (and by
    which PMT: n x 16), the expectation the sampled ids estimate."""
    pos = np.asarray(positions, np.float64).reshape(-1, 3)
    wl = np.asarray(wavelengths, np.float64)
    rel = (pos - np.asarray(target["position"], float)) / float(target["radius"])
    acc = [np.interp(wl, model["acc_wavelength"], model["acc_group1"], left=0, right=0),
           np.interp(wl, model["acc_wavelength"], model["acc_group2"], left=0, right=0)]
    out = np.zeros((len(wl), 16))
    for k in range(16):
        pt = np.arccos(np.clip(rel @ np.asarray(model["pmt_dir"][k], float), -1, 1))
        g = int(model["pmt_group"][k])
        sig = model["sigma_group1"] if g == 1 else model["sigma_group2"]
        pdf = pt / sig ** 2 * np.exp(-pt ** 2 / (2 * sig ** 2))
        s = np.sin(pt)
        with np.errstate(divide="ignore", invalid="ignore"):
            w = np.where(s != 0, pdf / (0.5 * s), 0.0)
        out[:, k] = w * acc[g - 1] / 8
    return out
