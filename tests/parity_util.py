"""Helpers shared by the GPU parity tests: moving an oracle state into a GPU engine, pairing the
two engines' interaction records, and per-contact relative force errors."""
import numpy as np


def by_pair(recs):
    return {(int(r[0]), int(r[1])): r for r in recs}


def snapshot_into(eng, orc, force_collider=False, periodic=False):
    eng.put_body_state(orc.bodies())
    eng.put_interactions(orc.interactions())
    s = orc.scalars()
    if force_collider:
        s = s.copy()
        s[1] = 2.0
        orc.set_scalars(s)
    eng.put_scalars(s)
    if periodic:
        eng.put_cell(orc.cell())


def touching_common(gi, ri):
    G, R = by_pair(gi), by_pair(ri)
    keys = [k for k, r in R.items() if k in G and r[4] > 0 and r[2] == 1]
    return np.array([G[k] for k in keys]), np.array([R[k] for k in keys]), keys


def rel_force_errors(G, R):
    """|F_gpu - F_oracle| / |F_oracle| per contact, F = normal + shear force."""
    fg = G[:, 26:29] + G[:, 29:32]
    fr = R[:, 26:29] + R[:, 29:32]
    den = np.linalg.norm(fr, axis=1)
    return np.linalg.norm(fg - fr, axis=1) / np.where(den > 0, den, 1)
