"""The me2j interaction file format (read by read_me2j_interaction, src/interaction_IO.f90:282-400).

A gzipped text file: one header line, then the record values, ten per line, the first in
an f12.7 field and the others in f13.7 fields (the last line shorter).  Values come in the
record order of the reference's loop, four per record: T=0, then T=1 with Mt = -1, 0, +1.
`Engine.me2j_to_slab` turns them into the proton-neutron J-scheme arrays.
"""
from __future__ import annotations

import gzip

import numpy as np


def read_me2j(path: str) -> np.ndarray:
    """All record values of a (gzipped) me2j file, parsed with the fixed field widths."""
    opener = gzip.open if str(path).endswith(".gz") else open
    vals = []
    with opener(path, "rt") as f:
        f.readline()  # header
        for line in f:
            line = line.rstrip("\n")
            if not line.strip():
                continue
            vals.append(float(line[:12]))
            for k in range(12, len(line), 13):
                field = line[k:k + 13]
                if field.strip():
                    vals.append(float(field))
    return np.array(vals)


def write_me2j(path: str, values: np.ndarray, header: str = "synthetic me2j") -> None:
    """Write record values in the me2j layout (gzipped when the name ends in .gz)."""
    opener = gzip.open if str(path).endswith(".gz") else open
    v = np.asarray(values, dtype=np.float64)
    with opener(path, "wt") as f:
        f.write(header + "\n")
        for i in range(0, v.size, 10):
            row = v[i:i + 10]
            f.write(f"{row[0]:12.7f}" + "".join(f"{x:13.7f}" for x in row[1:]) + "\n")
