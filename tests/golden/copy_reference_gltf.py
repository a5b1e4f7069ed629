"""Copies the reference's Cornell-box glTF fixture (scenes/cornell_box.gltf and .bin of the
reference project) unchanged into tests/golden/ and prints their SHA-256, which
tests/test_gltf.py checks.  Run where the reference project is available:

    python tests/golden/copy_reference_gltf.py /path/to/reference

The files are scene data (32 triangles, one emissive quad of strength 40, a metal box); they
are committed byte for byte so that the importer and the GPU render of an imported scene are
tested on the reference's own input on any machine.
"""
import hashlib
import shutil
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def main(reference_root: str) -> None:
    for name in ("cornell_box.gltf", "cornell_box.bin"):
        src = Path(reference_root) / "scenes" / name
        dst = HERE / name
        shutil.copyfile(src, dst)
        print(name, hashlib.sha256(dst.read_bytes()).hexdigest())


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
