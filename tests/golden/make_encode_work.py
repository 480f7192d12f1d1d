"""Writes encode_work.json: the algorithmic work of the benchmark's DXT1 encode workload (the
1024 x 1024 texture of seed 100 with its 11 box-filtered levels, perceptual metric, 3-colour blocks
allowed, Uber quality), counted by the oracle -- the CPU restatement pinned bit-exactly to the
reference -- as the candidate x unique-colour evaluations the reference's evaluate_solution loops
make (crnlib/crn_dxt1.cpp:1370-1592). The GPU encoder's roofline divides this fixed count (times
the lane-ops of one evaluation) by its kernel time.
Run:  python tests/golden/make_encode_work.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from crunch2_gb300 import texgen  # noqa: E402
from oracle import port  # noqa: E402


def main() -> None:
    levels = texgen.mip_chain(texgen.colour_texture(1024, 1024, 100))
    blocks = np.concatenate([texgen.image_blocks(l) for l in levels])
    evals = port.dxt1_count_evaluations(blocks, True, True, threads=os.cpu_count() or 4)
    out = {"workload": "1024x1024 texture, seed 100, 11 box-filtered levels", "blocks": int(blocks.shape[0]),
           "texels": int(sum(l.shape[0] * l.shape[1] for l in levels)), "perceptual": True,
           "use_alpha_blocks": True, "quality": "uber", "candidate_colour_evaluations": evals}
    with open(os.path.join(HERE, "encode_work.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
    print(out)


if __name__ == "__main__":
    main()
