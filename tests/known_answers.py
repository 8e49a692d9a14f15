"""Known-answer constants of the reference's own tests (extracted by
tests/golden/make_golden.py into tests/golden/reference_known_answers.json)
and the Sedov known-answer run shared by the oracle and GPU tests."""
import json
import os

import numpy as np

KA = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                 "reference_known_answers.json")))


def sedov_known_answer_run(stepper, cfg, x, v, B):
    """Run the Sedov test to tmax with global timesteps (evolve_utils.F90:91-100:
    dt = min(dtforce, dtcourant, dterr, time left to the output); returns the
    relative total-energy change and the largest momentum component."""
    m = cfg["massoftype"]
    tmax = KA["sedov_tmax"]["value"]

    def energy(vv):
        return float(np.sum(0.5 * m * np.sum(vv[:, :3] ** 2, axis=1)) + np.sum(m * vv[:, 3]))

    dt, get = stepper
    e0 = energy(v)
    t = 0.0
    nsteps = 0
    while t < tmax * (1.0 - 1.0e-12):
        dt = min(dt, tmax - t)
        dtn, _, dterr = get.step(t, dt)
        t += dt
        nsteps += 1
        dt = min(dtn, dterr)
    xo, vo, _ = get.download() if hasattr(get, "download") else get.get_particles()
    mom = float(np.abs(np.sum(m * vo[:, :3], axis=0)).max())
    return abs(energy(vo) / e0 - 1.0), mom, nsteps, xo, vo
