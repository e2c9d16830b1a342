"""director2data: the oracle against the reference's own output
(``tests/golden/director.npz``: seeded directors of lengths 0 to 1.3, default
parameters and a masked host region with a scale factor), within 1e-15."""
import os

import numpy as np

import dtmm_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


def test_oracle_director2data_matches_reference():
    z = np.load(os.path.join(HERE, "golden", "director.npz"))
    th, ev, ea = O.director2data(z["director"])
    assert np.array_equal(th, z["thickness_default"])
    assert np.abs(ev - z["epsv_default"]).max() < 1e-15 * 4
    assert np.abs(ea - z["epsa_default"]).max() < 1e-15 * 4
    _, ev, ea = O.director2data(z["director"], mask=z["mask"], no=1.52, ne=1.71, nhost=1.4, scale_factor=0.8)
    assert np.abs(ev - z["epsv_masked"]).max() < 1e-15 * 4
    assert np.abs(ea - z["epsa_masked"]).max() < 1e-15 * 4
