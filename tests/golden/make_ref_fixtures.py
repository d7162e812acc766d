"""Record the reference's own outputs as golden vectors.

Needs a GB300 and the cubins built by oracle/build_ref.sh from the reference's
sources (they travel with the checkout; the reference tree itself is not needed
here).  Inputs are the seeded synthetic perambulator / elementals below at the
reference's only supported size, Nev = 100, with Nt = 2; they are regenerated
by the tests from the same seeds.  Output: one compressed .npz with the per-row
kernel outputs and the host-reduced correlators of every diagram family.

    python tests/golden/make_ref_fixtures.py [--out tests/golden/ref_outputs.npz]
"""

import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

NEV, NT = 100, 2
SEED = 2024


def inputs():
    from contractions_code_scattering_gb300 import synth
    prop = synth.make_prop(NT, NEV, seed=SEED, decay=0.35)
    rng = np.random.default_rng(SEED + 1)
    mom5 = np.stack([synth.make_phi_hermitian(NT, NEV, seed=SEED + 2)] +
                    [synth.make_phi_random(NT, NEV, rng) for _ in range(4)], axis=1)
    p = [synth.make_phi_random(NT, NEV, rng) for _ in range(4)]
    mom2 = np.stack([synth.make_phi_random(NT, NEV, rng) for _ in range(2)], axis=1)
    return dict(prop=prop, mom5=np.ascontiguousarray(mom5), p1=p[0], p2=p[1], p3=p[2], p4=p[3],
                mom2=np.ascontiguousarray(mom2))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(ROOT, "tests", "golden", "ref_outputs.npz"))
    args = ap.parse_args()
    from oracle import refkernels as R
    d = inputs()
    out = {}
    out["rho_rows"], out["rho_corr"] = R.rho(d["prop"], d["mom5"])
    out["sigma_rows"], out["sigma_corr"] = R.sigma(d["prop"], d["mom2"])
    out["loop_rows"], out["loop"] = R.loop_unity(d["prop"], d["p1"])
    for idir in range(3):
        out["rhopi%d_rows" % idir], out["rhopi%d_corr" % idir] = R.rhopi(d["prop"], d["p1"], d["p2"], d["mom5"], idir)
    for iso in (0, 1):
        res = R.pipi(d["prop"], d["p1"], d["p2"], d["p3"], d["p4"], iso)
        for k, v in res.items():
            out["pipi_I%d_%s" % (iso, k)] = v
    sp = R.sigmapi(d["prop"], d["p1"], d["p2"], d["mom2"])
    for k, v in sp.items():
        out["sigmapi_" + k] = v
    out["meta_nev_nt_seed"] = np.array([NEV, NT, SEED])
    np.savez_compressed(args.out, **out)
    print("wrote %d arrays to %s" % (len(out), args.out))


if __name__ == "__main__":
    main()
