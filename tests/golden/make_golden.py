"""Regenerate the golden vectors of this directory.

reference_primitives.json comes from oracle/_ref/ref_golden, a small driver
linked against the reference's own hash, PCG sampler, Box-Muller and
tangent-frame code compiled from the reference tree (oracle/Makefile, target
"ref").  It is only runnable where the reference tree is present; the JSON it
writes is committed so the tests never need the reference at run time.

    python tests/golden/make_golden.py --ref /path/to/reference   (or GPIS_REFERENCE=...)
"""
import argparse
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("GPIS_REFERENCE"))
    args = ap.parse_args()
    if not args.ref:
        ap.error("the reference tree is required: --ref <path> or GPIS_REFERENCE")
    subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={args.ref}"])
    out = subprocess.check_output([os.path.join(ROOT, "oracle", "_ref", "ref_golden")])
    doc = json.loads(out)
    doc["_about"] = ("Generated by tests/golden/make_golden.py from the reference's own "
                     "MathUtil.hpp, UniformSampler.hpp, Gaussian.cpp and TangentFrame.hpp "
                     "(compiled by g++ on x86-64). Floats are uint32 bit patterns; doubles "
                     "are uint64 bit patterns as strings.")
    path = os.path.join(HERE, "reference_primitives.json")
    with open(path, "w") as f:
        json.dump(doc, f, indent=0, sort_keys=True)
        f.write("\n")
    print(f"wrote {path}", file=sys.stderr)


if __name__ == "__main__":
    main()
