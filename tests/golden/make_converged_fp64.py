"""Generates stage_converged_fp64.json: the FP64 oracle (the reference's LOOP
restated in C++ and instantiated on double, the stand-in for the reference
built with -fdefault-real-8) marched from SETUP's initial guess on the
single-stage turbine (65 x 242 x 49, SFXIN = SFTIN = 0.02) until the
reference's own end test holds (multall-open-18.3.f:3762-3764: EAVG < CONLIM
and ECONT < 0.01, or |EMAX| < 4 CONLIM and ECONT < 0.01; CONLIM = 1e-5) or
MAXSTEPS steps have run.  It records the mass flows and efficiencies at the
stop, and the same every 1000 steps, as the fixture that the convergence
bench and tests measure the GPU paths against (|eta - eta_FP64| <= 1e-4,
mass flow within 1e-4 relative).

It runs for about half an hour on one x86 core.  From the repository root:
    python tests/golden/make_converged_fp64.py
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "multall-open-18.3_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from mgpu import case, common_setup  # noqa: E402
import oracle as O  # noqa: E402

MAXSTEPS = 20000
SMOOTHING = 0.02


def spec():
    sp = case.turbine_stage()
    sp.sfxin = sp.sftin = SMOOTHING
    return sp


def main():
    cd = common_setup.build_common(spec())
    cd.ints["NSTEPS_MAX"] = MAXSTEPS
    o = O.Oracle(cd, double=True)
    o.setup_calls()
    hist = []
    t0 = time.time()
    m = None
    for n in range(1, MAXSTEPS + 1):
        m = o.step()
        if n % 1000 == 0 or m.ifend:
            r = o.integrals()
            hist.append({"nstep": m.nstep, "eavg": m.eavg, "emax": m.emax, "econt": m.econt,
                         "eta_tt": r.eta_tt, "eta_ts": r.eta_ts, "mass_flow_in": r.mass_flow_in,
                         "mass_flow_out": r.mass_flow_out})
            print(json.dumps(hist[-1]), f"{time.time() - t0:.0f}s", flush=True)
        if m.ifend:
            break
    r = o.integrals()
    out = {"case": "turbine_stage 65x242x49, SFXIN=SFTIN=0.02, CONLIM=1e-5", "oracle": "FP64",
           "stopped_by_end_test": bool(m.ifend and m.nstep < MAXSTEPS), "nstep": m.nstep,
           "eavg": m.eavg, "emax": m.emax, "econt": m.econt,
           "eta_tt": r.eta_tt, "eta_ts": r.eta_ts, "mass_flow_in": r.mass_flow_in,
           "mass_flow_out": r.mass_flow_out, "po_ratio": r.po_ratio, "to_ratio": r.to_ratio,
           "history": hist}
    with open(os.path.join(HERE, "stage_converged_fp64.json"), "w") as f:
        json.dump(out, f, indent=1)
    o.close()


if __name__ == "__main__":
    main()
