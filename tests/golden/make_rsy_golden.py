"""Writes the .rsy golden fixtures of tests/test_rsy.py with the reference's own
code: oracle/ref_rsy/Makefile builds oracle/_ref/rsy_writer from the
reference's src/Asset/Asset.cpp (asset::write and asset::read, unchanged);
the writer fills an asset from a seed, writes it with asset::write, reads it
back with asset::read and prints what that reader decoded. Each fixture is the
.rsy file and that JSON. Needs the reference's sources (set REF to its src/
directory); the fixtures themselves are committed.

    REF=/root/reference/src python tests/golden/make_rsy_golden.py
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CASES = [(1, 1), (2, 2), (3, 3)]  # (seed, meshes)


def main() -> None:
    ref = os.environ.get("REF", "/root/reference/src")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref_rsy"), f"REF={ref}"], check=True)
    writer = os.path.join(ROOT, "oracle", "_ref", "rsy_writer")
    out_dir = os.path.join(HERE, "rsy")
    os.makedirs(out_dir, exist_ok=True)
    for seed, meshes in CASES:
        stem = os.path.join(out_dir, f"ref_s{seed}_m{meshes}")
        r = subprocess.run([writer, stem + ".rsy", str(seed), str(meshes)], check=True, capture_output=True, text=True)
        with open(stem + ".json", "w") as f:
            f.write(r.stdout)
        print(stem, os.path.getsize(stem + ".rsy"), "bytes")


if __name__ == "__main__":
    sys.exit(main())
