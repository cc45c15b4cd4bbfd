"""Generates deck_converged_fp64.json: the FP64 oracle (the reference's LOOP
restated in C++ on double) marched on the reference's own single-stage
turbine deck (tests/golden/decks/Single-stage-turbine-17.1.npz, as the deck
reader leaves it) from SETUP's initial guess for the deck's NSTEPS_MAX
steps.  It records the first step at which the deck's own end test holds
(multall-open-18.3.f:3762-3764 with the deck's CONLIM; the march goes on
past it), and the monitors, mass flows and efficiencies at the end.  The GPU
test checks that the library meets the end test at nearly the same step,
and that after NSTEPS_MAX steps its mass flows and efficiency are within
1e-4 of these.

From the repository root (about half an hour on one x86 core):
    python tests/golden/make_deck_converged_fp64.py
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "multall-open-18.3_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from mgpu import common_setup, deck  # noqa: E402
import oracle as O  # noqa: E402

NAME = "Single-stage-turbine-17.1"


def main():
    spec, geo = deck.load_fixture(os.path.join(HERE, "decks", NAME + ".npz"))
    cd = common_setup.build_common(spec, geo)
    conlim = cd.reals["CONLIM"]
    nsteps = cd.ints["NSTEPS_MAX"]
    cd.reals["CONLIM"] = 0.0                # march on past the end test
    cd.ints["NSTEPS_MAX"] = 10 ** 9
    o = O.Oracle(cd, double=True)
    o.setup_calls()
    hist = []
    t0 = time.time()
    end_step = None
    for n in range(1, nsteps + 1):
        m = o.step()
        if end_step is None and n % 5 == 0 and m.econt < 0.01 and (m.eavg < conlim or abs(m.emax) < 4 * conlim):
            end_step = n
        if n % 500 == 0 or n == end_step:
            r = o.integrals()
            hist.append({"nstep": n, "eavg": m.eavg, "emax": m.emax, "econt": m.econt, "eta_tt": r.eta_tt,
                         "mass_flow_in": r.mass_flow_in, "mass_flow_out": r.mass_flow_out})
            print(json.dumps(hist[-1]), f"{time.time() - t0:.0f}s", flush=True)
    r = o.integrals()
    out = {"deck": NAME + ".dat", "oracle": "FP64", "conlim": conlim, "nsteps_max": nsteps,
           "end_test_step": end_step, "nstep": nsteps, "eavg": m.eavg, "emax": m.emax, "econt": m.econt,
           "eta_tt": r.eta_tt, "eta_ts": r.eta_ts, "mass_flow_in": r.mass_flow_in, "mass_flow_out": r.mass_flow_out,
           "history": hist}
    with open(os.path.join(HERE, "deck_converged_fp64.json"), "w") as f:
        json.dump(out, f, indent=1)
    o.close()


if __name__ == "__main__":
    main()
