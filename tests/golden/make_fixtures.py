"""Copies the reference's test vectors for this path into tests/golden/ and pins
the oracle's decoded output for each of them.

Run from the repository root with the reference checked out at REFERENCE
(default /root/reference):

    python tests/golden/make_fixtures.py

Each copied file is checked against the SHA-256 recorded in the reference's
own manifests (testdata/manifests/jpeg.toml, testdata/manifests/y4m.toml,
testdata/dv/valid/SHA256SUMS). The oracle checksums (SHA-256 of every decoded
plane, plus status and message) go to oracle_outputs.json; tests compare the
oracle against it so any later change to the oracle is visible.
"""

from __future__ import annotations

import hashlib
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REFERENCE = os.environ.get("REFERENCE", "/root/reference")

FILES = [
    "jpeg/valid/baseline-420.jpg",
    "jpeg/valid/minimal-gray.jpg",
    "jpeg/valid/unknown-app-marker.jpg",
    "jpeg/valid/restart-interval.jpg",
    "jpeg/parser/stuffed-restarts.jpg",
    "jpeg/invalid/invalid-length.jpg",
    "jpeg/invalid/missing-eoi.jpg",
    "jpeg/invalid/truncated-marker.jpg",
    "jpeg/encoded/mmrecode-q85-420.mjpg",
    "y4m/valid/two-frame-420.y4m",
    "dv/valid/dv25-525-60-one-frame.dv",
    "dv/valid/dv25-625-50-one-frame.dv",
]


def manifest_hashes() -> dict:
    hashes = {}
    for name in ("jpeg.toml", "y4m.toml"):
        text = open(os.path.join(REFERENCE, "testdata", "manifests", name)).read()
        for path, digest in re.findall(r'path = "([^"]+)".*?sha256 = "([0-9a-f]+)"', text, re.S):
            hashes[path] = digest
    for line in open(os.path.join(REFERENCE, "testdata", "dv", "valid", "SHA256SUMS")):
        digest, path = line.split()
        hashes["dv/valid/" + os.path.basename(path)] = digest
    return hashes


def main() -> int:
    hashes = manifest_hashes()
    for rel in FILES:
        src = os.path.join(REFERENCE, "testdata", rel)
        data = open(src, "rb").read()
        digest = hashlib.sha256(data).hexdigest()
        if hashes.get(rel) != digest:
            print(f"{rel}: SHA-256 {digest} does not match the reference manifest {hashes.get(rel)}")
            return 1
        dst = os.path.join(HERE, rel)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        shutil.copyfile(src, dst)
    sys.path.insert(0, ROOT)
    import oracle

    outputs = {}
    for rel in FILES:
        data = open(os.path.join(HERE, rel), "rb").read()
        if rel.startswith("jpeg/"):
            r = oracle.jpeg_decode(data)
        elif rel.startswith("dv/"):
            r = oracle.dv_decode(data)
        else:
            continue
        entry = {"status": r.status, "message": r.message}
        if r.frame:
            entry["format"] = r.frame.format
            entry["planes"] = [[w, h, hashlib.sha256(b).hexdigest()] for w, h, b in r.frame.planes]
            entry["rgb24"] = hashlib.sha256(oracle.rgb24(r.frame)).hexdigest()
        outputs[rel] = entry
    with open(os.path.join(HERE, "oracle_outputs.json"), "w") as f:
        json.dump(outputs, f, indent=1, sort_keys=True)
    print("wrote", len(FILES), "fixtures and oracle_outputs.json")
    return 0


if __name__ == "__main__":
    sys.exit(main())
