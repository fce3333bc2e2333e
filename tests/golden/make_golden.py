"""Generate the golden hit-record fixtures from the reference itself.

Runs the reference's own device programs and scene code (cuda/sun.cu, cuda/intersection.cu,
cuda/materials.cu, lib/element.cpp, lib/Aperture.cpp), built on the host by `make -C oracle ref`
under the project's OptiX/cuRAND stand-ins, on small seeded cases, and stores their hit records,
element ids, device geometry and sun plane as compressed .npz files next to this script.

Usage (needs the reference sources):
    CSP_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from tests.golden.cases import CASES  # noqa: E402


def main():
    oracle.build(with_ref=True)
    ref = oracle.RefHost()
    for name, make in CASES.items():
        sc, n, seed, instance, first = make()
        hits, ids = ref.trace(sc.elements, sc.sun_dir, sc.sun_param, first_ray=first, count=n, seed=seed,
                              instance=instance)
        prims, sun = ref.scene_info(sc.elements, sc.sun_dir, sc.sun_param)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), hits=hits.astype(np.float32), ids=ids,
                            prims=prims, sun=sun, elements=sc.elements, sun_dir=sc.sun_dir,
                            sun_param=np.float64(sc.sun_param), seed=np.uint64(seed),
                            instance=np.uint32(instance), first=np.uint64(first))
        st = hits[:, :, 0]
        print(f"{name}: {n} rays from {first}, mirror hits {int((st == 1).sum())}, receiver hits {int((st == 2).sum())}")


if __name__ == "__main__":
    main()
