"""Set-ups restated from the reference's examples (CPU)."""

import numpy as np


def test_homogeneous_box_reproduces_reference_count():
    """The reference's homogeneous benchmark at 2^25 target particles runs on 33,848,064
    particles (its published single-GPU result files); the restated HCP set-up must give
    that exact count, inside the periodic box the lattice closes."""
    from shamrock_gb300 import setups

    s = setups.homogeneous_box(1 << 25)
    assert len(s["h"]) == 33848064
    lo, hi = np.asarray(s["box_min"]), np.asarray(s["box_max"])
    assert np.all(s["pos"] >= lo) and np.all(s["pos"] < hi)
    # total injected energy sum m u ~ 1 (u_inj W(r, 16 dr) integrates to u_inj)
    assert abs(s["pmass"] * s["u"].sum() - 1.0) < 0.02
