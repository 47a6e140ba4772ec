"""The reference's model files (``tests/golden/ref_model_assets.npz``, recorded
byte for byte by ``tests/golden/make_golden.py``) written back to disk, so the
tests load them through the package's own loaders and model search path.

The cylinder is "Cylinder" by username7777777
(https://sketchfab.com/3d-models/cylinder-679440db551840d2b4586e790228a12c),
licensed under CC-BY-4.0 (http://creativecommons.org/licenses/by/4.0/); the
cone is part of the reference (MIT licence)."""
import os

import numpy as np

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_model_assets.npz")


def facts() -> dict:
    d = np.load(FIXTURE)
    return {k: d[k] for k in d.files}


def unpack(dst: str) -> str:
    """Write ``models/cone.egg`` and ``models/cylinder/{scene.gltf, scene.bin,
    license.txt}`` under ``dst``; returns ``dst`` (a model search path entry)."""
    d = np.load(FIXTURE)
    files = {"models/cone.egg": "cone_egg", "models/cylinder/scene.gltf": "cylinder_gltf",
             "models/cylinder/scene.bin": "cylinder_bin", "models/cylinder/license.txt": "cylinder_license"}
    for rel, key in files.items():
        path = os.path.join(dst, rel)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "wb") as f:
            f.write(d[key].tobytes())
    return dst
