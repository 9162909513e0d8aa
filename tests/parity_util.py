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


def oracle_state(orc, periodic=False):
    """What restore_oracle needs to repeat the oracle's next step from here."""
    return (orc.bodies(), orc.interactions(), orc.scalars(), orc.cell() if periodic else None)


def restore_oracle(spec, state, threads=1, periodic_fix=False):
    from oracle import OracleScene
    bodies, intr, sc, cell = state
    o = OracleScene.from_spec(spec, threads=threads)
    if periodic_fix:
        o.set_periodic_fix(True)
    o.set_bodies(bodies)
    o.set_interactions(intr)
    o.set_scalars(sc)
    if cell is not None:
        o.put_cell(cell)
    o.rebuild_sorted_bounds()
    return o


def oracle_spread(spec, state, seeds=(1, 2, 3), rel=0.0, threads=1, periodic_fix=False):
    """The reference's own conditioning, per touching pair: the largest relative change of the
    contact force (normal + shear) of the next step when the narrowphase's pow/sin/cos/atan2
    results move in their last bits (oracle.set_math_noise: one ulp for rel = 0, else rel times
    the value), over a few noise seeds.  Returns {pair: spread}."""
    import oracle
    ref = restore_oracle(spec, state, threads, periodic_fix)
    ref.step(1)
    R = by_pair(ref.interactions())
    out = {k: 0.0 for k, r in R.items() if r[4] > 0 and r[2] == 1}
    try:
        for s in seeds:
            oracle.set_math_noise(s, rel)
            o = restore_oracle(spec, state, threads, periodic_fix)
            o.step(1)
            N = by_pair(o.interactions())
            for k in out:
                n = N.get(k)
                fr = R[k][26:29] + R[k][29:32]
                den = np.linalg.norm(fr)
                if n is None or not (n[4] > 0 and n[2] == 1):
                    out[k] = np.inf
                    continue
                fn = n[26:29] + n[29:32]
                out[k] = max(out[k], float(np.linalg.norm(fn - fr) / (den if den > 0 else 1)))
    finally:
        oracle.set_math_noise(0)
    return out
