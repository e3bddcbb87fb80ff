"""Pack the tabulated symmetric spherical designs into ``sphere_designs.npz``.

The designs are R. S. Womersley's published symmetric spherical t-designs
(antipodally symmetric point sets on S^2).  The reference solver ships them as
text tables under ``src/collision/spherical_design/symmetric/`` and selects one
by point count (``src/collision/spherical_design/__init__.py:62-88``).  The
quadrature points must be identical for operator parity, so this script reads
those tables once and stores them as float64 arrays keyed ``m{npts:05d}``
(with the design strength in ``qdeg_m{npts:05d}``).  Run it where the reference
checkout is present (``PII_REFERENCE_ROOT``, required); the package reads
only the ``.npz``:

    PII_REFERENCE_ROOT=<reference checkout> python tests/golden/make_designs.py
"""
import os
import re
import sys

import numpy as np

OUT = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                   "proj-int-inelastic_gb300", "data", "sphere_designs.npz")


def main(out=OUT):
    root = os.environ.get("PII_REFERENCE_ROOT")
    if not root:
        raise SystemExit("set PII_REFERENCE_ROOT to the reference checkout (the directory holding src/)")
    SRC = os.path.join(root, "src/collision/spherical_design/symmetric")
    arrays = {}
    for name in sorted(os.listdir(SRC)):
        m = re.match(r"womersley-ss(\d+)-m(\d+)\.txt$", name)
        if not m:
            continue
        pts = np.loadtxt(os.path.join(SRC, name), dtype=np.float64).reshape(-1, 3)
        npts = int(m.group(2))
        assert pts.shape[0] == npts, name
        arrays[f"m{npts:05d}"] = pts
        arrays[f"qdeg_m{npts:05d}"] = np.array(int(m.group(1)))
    np.savez(out, **arrays)
    print(f"wrote {out}: {sorted(k for k in arrays if not k.startswith('qdeg'))}")


if __name__ == "__main__":
    main(*sys.argv[1:])
