"""Loading of the reference-generated fixtures in tests/golden/."""
import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files if k != "meta"}
    d["meta"] = json.loads(str(z["meta"]))
    return d


def incr(meta):
    n, skip = meta["ntimesteps"], meta["skip"] or 1
    return 1.0 / (n // skip) if n // skip > 0 else 1.0


GOLDEN_MSD = os.path.join(GOLDEN, "msd")


def msd_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_MSD, "*.npz")))


def load_msd(name):
    z = np.load(os.path.join(GOLDEN_MSD, name + ".npz"))
    d = {k: z[k] for k in z.files if k != "meta"}
    d["meta"] = json.loads(str(z["meta"]))
    return d


GOLDEN_NEIGH = os.path.join(GOLDEN, "neigh")


def neigh_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_NEIGH, "*.npz")))


def load_neigh(name):
    z = np.load(os.path.join(GOLDEN_NEIGH, name + ".npz"))
    d = {k: z[k] for k in z.files if k != "meta"}
    d["meta"] = json.loads(str(z["meta"]))
    return d


def neigh_entries(d):
    """{(atom, type): (indices, rows)} of a neighbour fixture."""
    out, p = {}, 0
    N, nt = d["sizes"].shape
    for a in range(N):
        for k in range(nt):
            n = int(d["sizes"][a, k])
            out[a, k] = (d["idx"][p:p + n], d["rows"][p:p + n])
            p += n
    return out
