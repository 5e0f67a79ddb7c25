"""Copies the reference's example input folders (examples/{test1,test2,test3,test4,Altyn}/input/*.dat)
into tests/golden/inputs/<case>/ as fixtures for the input parser and the program tests.

Only the text inputs are copied, byte for byte.  The reference builds each example's Vp/Vs SU
models with a MATLAB script (examples/test*/input/create_*.m) and ships no model files (Altyn's
smoothed models are among its missing large files); tests/example_models.py writes them instead.

Run once where the reference tree is present:  python tests/golden/make_inputs.py [REFROOT]
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ("test1", "test2", "test3", "test4", "Altyn")


def main(refroot):
    for case in CASES:
        src = os.path.join(refroot, "examples", case, "input")
        dst = os.path.join(HERE, "inputs", case)
        os.makedirs(dst, exist_ok=True)
        for name in sorted(os.listdir(src)):
            if name.endswith(".dat"):
                shutil.copyfile(os.path.join(src, name), os.path.join(dst, name))
                os.chmod(os.path.join(dst, name), 0o644)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REFROOT", "/root/reference"))
