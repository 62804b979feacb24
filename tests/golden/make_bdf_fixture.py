"""Generate tests/golden/ref_generator_bending_320.bdf with the reference's own
mesh generator (tools/generate_chexa_mesh.py of vibestran), so that the
native BDF reader is pinned on the reference's deck conventions (free-field
cards, '+' CHEXA continuations, %.6E numbers, SPC1 THRU, comments) without a
copy of the reference at test time.  Run in a container that has the
reference checked out:
    python tests/golden/make_bdf_fixture.py <reference root>
    (or with VSGB_REFERENCE_ROOT set in the environment)
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VSGB_REFERENCE_ROOT")
    if not ref:
        raise SystemExit("usage: make_bdf_fixture.py <reference root> "
                         "(or set VSGB_REFERENCE_ROOT)")
    gen = os.path.join(ref, "tools", "generate_chexa_mesh.py")
    out = os.path.join(HERE, "ref_generator_bending_320.bdf")
    subprocess.run([sys.executable, gen, "320", "--load-case", "bending", "-o", out], check=True)
    print("wrote", out)


if __name__ == "__main__":
    main()
