"""Extract the ndec=40 digital Hankel filter taps used by the anomaly-to-anomaly
Green-tensor build and write them as data files for this package.

The reference loads the taps at run time from its resource file
``Extreme.Cartesian/Resources/hankelcoeff.xml`` (``HankelCoefficients.LoadN40``,
``Extreme.Cartesian/Green/Scalar/Impl/HankelCoefficients.cs:37-65``). The taps are
a published numeric table, so they have to be identical for parity: this script
copies the ``ndec="40"`` set (431 J0 taps ``h0`` and 431 J1 taps ``h1``) into

* ``hankel_ndec40.npz``  -- read by the Python side and by the tests;
* ``../csrc/hankel_ndec40.inc`` -- compiled into ``libegx.so``.

Run it once in a checkout that has the reference tree beside it:

    python extreme_gb300/data/make_hankel_table.py /path/to/reference
"""
import os
import sys
import xml.etree.ElementTree as ET

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load(ref_root, ndec="40"):
    path = os.path.join(ref_root, "Extreme.Cartesian", "Resources", "hankelcoeff.xml")
    root = ET.parse(path).getroot()
    for coeffs in root.findall("Coefficients"):
        if coeffs.get("ndec") == ndec:
            h0 = np.array([float(l.get("h0")) for l in coeffs.findall("line")])
            h1 = np.array([float(l.get("h1")) for l in coeffs.findall("line")])
            return h0, h1
    raise KeyError(ndec)


def main():
    # the reference checkout: argument, else EGX_REFERENCE, else "reference" beside this checkout
    beside = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(HERE))), "reference")
    ref_root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("EGX_REFERENCE", beside)
    h0, h1 = load(ref_root)
    assert h0.size == 431 and h1.size == 431
    np.savez(os.path.join(HERE, "hankel_ndec40.npz"), h0=h0, h1=h1,
             ndec=np.int32(40), l1=np.int32(-300), l2=np.int32(130))
    inc = os.path.join(HERE, "..", "csrc", "hankel_ndec40.inc")
    with open(inc, "w") as f:
        f.write("// Generated by extreme_gb300/data/make_hankel_table.py: ndec=40 "
                "digital Hankel filter taps (431 J0 taps, 431 J1 taps).\n")
        f.write("static const double kHankelJ0[431] = {\n")
        f.write(",\n".join(repr(float(v)) for v in h0))
        f.write("};\nstatic const double kHankelJ1[431] = {\n")
        f.write(",\n".join(repr(float(v)) for v in h1))
        f.write("};\n")
    print("wrote", h0.size, "taps")


if __name__ == "__main__":
    main()
