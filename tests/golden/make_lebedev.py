"""Writes lebedev_rules.json: the Lebedev-Laikov angular rules of 6, 14, 26,
110, 170, 194, 302, 590 and 770 points (x, y, z, weight summing to 1), from
scipy.integrate.lebedev_rule (scipy >= 1.15), for the oracle's molecular
meshes and basin integrals (rays and beta spheres).  Run from this directory: python make_lebedev.py"""
import json

import numpy as np
from scipy.integrate import lebedev_rule

out = {}
for n, deg in ((6, 3), (14, 5), (26, 7), (110, 17), (170, 21), (194, 23), (302, 29), (590, 41), (770, 47)):
    x, w = lebedev_rule(deg)
    assert x.shape[1] == n
    out[str(n)] = [[float(a), float(b), float(c), float(v / (4.0 * np.pi))] for (a, b, c), v in zip(x.T, w)]
with open("lebedev_rules.json", "w") as fh:
    json.dump(out, fh)
