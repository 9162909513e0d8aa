"""Writes tests/golden/compression_stats.json: the CPU oracle's results of config 1's periodic
compression to 100 kPa (tests/compression_protocol.py) and of config 2's servo-controlled
specimen (tests/servo_protocol.py) for seeds 1-5, and for the same seeds with a planted mistake
(contact stiffness kn x 1.3, so stresses at a given strain are 30% higher), which the
statistics test must tell apart from the correct oracle.

Run: python tests/golden/make_compression_stats.py [threads]   (about an hour on 8 cores; keys already
present in the file are kept, so a partial run resumes)
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.dirname(HERE)]

SEEDS = (1, 2, 3, 4, 5)
OUT = os.path.join(HERE, "compression_stats.json")


def run(seed, kn, threads):
    from oracle import OracleScene
    import compression_protocol as CP
    spec = CP.spec_for(seed, kn=kn)
    o = OracleScene.from_spec(spec, threads=threads)
    o.set_periodic_fix(True)
    r = CP.Run(spec, o)
    t0 = time.time()
    while True:
        r.advance()
        if r.check():
            break
    r.result["seconds"] = time.time() - t0
    return r.result


def run_servo(seed, kn, threads):
    from oracle import OracleScene
    import servo_protocol as SP
    spec, cfg = SP.spec_and_config(seed, kn=kn)
    o = OracleScene.from_spec(spec, threads=threads)
    r = SP.Run(spec, o, cfg)
    t0 = time.time()
    while True:
        r.advance()
        if r.check():
            break
    r.result["seconds"] = time.time() - t0
    return r.result


def main():
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else os.cpu_count()
    out = json.load(open(OUT)) if os.path.exists(OUT) else {}
    jobs = [(f"{label}/{seed}", fn, seed, kn) for fn, prefix in ((run, ""), (run_servo, "servo_"))
            for label, kn in ((prefix + "oracle", 1e5), (prefix + "oracle_kn_x1.3", 1.3e5)) for seed in SEEDS]
    for key, fn, seed, kn in jobs:
        if key in out:
            continue
        out[key] = fn(seed, kn, threads)
        print(key, out[key], flush=True)
        with open(OUT, "w") as f:
            json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
