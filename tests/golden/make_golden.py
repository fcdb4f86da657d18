"""Generate the golden fixtures in tests/golden from the reference's own code.

Runs the reference headers (oracle/_ref/libxref.so, built by
oracle/build_ref.py from the reference checkout) on small seeded scenes with
per-(pixel, sample) PCG streams and stores the radiance films, plus the
reference's vMF EM fit on the checker-masked hemisphere fixture of
Sandbox/VonMisesFisherDistribution/Main.cpp:66-82 (restated sample set, seeded
PCG). Usage: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.bindings import load_scene  # noqa: E402
from xitils_gb300 import scenes  # noqa: E402
from xitils_gb300.scene import NAIVE, IntegratorParams  # noqa: E402

CASES = {
    "cornell_48x48x4": (lambda: scenes.cornell(48, 48, 4), IntegratorParams()),
    "cornell_naive_32x32x4": (lambda: scenes.cornell(32, 32, 4), IntegratorParams(integrator=NAIVE)),
    "simple_path_tracer_48x48x4": (lambda: scenes.simple_path_tracer_scene(48, 48, 4), IntegratorParams()),
    "terrain_g65_40x40x2": (lambda: scenes.terrain(grid=65, width=40, height=40, spp=2, env_size=(128, 64)),
                            IntegratorParams()),
}


def main():
    out = {}
    for name, (make, params) in CASES.items():
        desc = make()
        ref = load_scene(desc, "reference")
        out[name] = ref.render_pcg(desc, params=params)
        print(name, float(out[name].mean()))
    np.savez_compressed(os.path.join(HERE, "reference_films.npz"), **out)


if __name__ == "__main__":
    main()
