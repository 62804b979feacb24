"""Copy the reference's own CHEXA8 end-to-end decks (tests/e2e/cases of
vibestran: chexa8_axial_force, chexa8_constrained_thermal, chexa8_free_thermal)
into tests/golden/ref_e2e/, so that the native BDF reader is pinned on them
on every machine, without a reference checkout at test time.  The decks are
test inputs of the reference, copied unchanged.

    python tests/golden/make_ref_decks.py <reference root>
    (or with VSGB_REFERENCE_ROOT set in the environment)
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DECKS = ("chexa8_axial_force", "chexa8_constrained_thermal", "chexa8_free_thermal")


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VSGB_REFERENCE_ROOT")
    if not ref:
        raise SystemExit("usage: make_ref_decks.py <reference root> "
                         "(or set VSGB_REFERENCE_ROOT)")
    out = os.path.join(HERE, "ref_e2e")
    os.makedirs(out, exist_ok=True)
    for name in DECKS:
        src = os.path.join(ref, "tests", "e2e", "cases", name + ".bdf")
        shutil.copyfile(src, os.path.join(out, name + ".bdf"))
        print("copied", src)


if __name__ == "__main__":
    main()
