"""Writes tests/golden/*.json from the reference's own golden result files.

Source: applications/integrationtests/mechanics/results/Brick8NStiffness.txt and
Brick8NInternalforce.txt of the NuTo project (legacy Python integration test Brick8N.py:18-82): one
Hex8 on [-1, 1]^3, E = 10, nu = 0.25, the four x = +1 nodes displaced by (0.2, 0.2, 0.2), 2x2x2 Gauss.

Run once where the reference tree is mounted:
    python tests/golden/make_golden.py /path/to/nuto
"""

import json
import os
import sys

import numpy as np


def main(ref_root):
    res = os.path.join(ref_root, "applications", "integrationtests", "mechanics", "results")
    K = np.loadtxt(os.path.join(res, "Brick8NStiffness.txt"), skiprows=1)
    f = np.loadtxt(os.path.join(res, "Brick8NInternalforce.txt"), skiprows=1)
    out = {
        "source": "applications/integrationtests/mechanics/results/Brick8N{Stiffness,Internalforce}.txt",
        "setup": {
            "coords": [[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                       [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]],
            "E": 10.0,
            "nu": 0.25,
            "displaced_nodes": [1, 2, 5, 6],
            "displacement": [0.2, 0.2, 0.2],
            "gauss_per_dir": 2,
        },
        "K_e": K.tolist(),
        "f_e": f.tolist(),
    }
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "brick8n.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
