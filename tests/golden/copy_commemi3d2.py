"""Copies the reference's COMMEMI3D2 example deck (model, project and the 40
anomaly-layer files of EndUser/ExtremeMt/Examples/COMMEMI3D2) into
tests/golden/commemi3d2 as a test fixture. The files are input data, copied
byte for byte.

    python tests/golden/copy_commemi3d2.py [REFERENCE_CHECKOUT]

The checkout defaults to EGX_REFERENCE, else a "reference" directory beside
this repository.
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    beside = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(HERE))), "reference")
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("EGX_REFERENCE", beside)
    src = os.path.join(ref, "EndUser", "ExtremeMt", "Examples", "COMMEMI3D2")
    dst = os.path.join(HERE, "commemi3d2")
    os.makedirs(dst, exist_ok=True)
    names = sorted(os.listdir(src))
    for name in names:
        shutil.copyfile(os.path.join(src, name), os.path.join(dst, name))
    print("copied %d files to %s" % (len(names), dst))


if __name__ == "__main__":
    main()
