"""Child process of the tuner tests (the tuner's memory is per process):
runs one calculation of a fixed seeded case with the kernel given on the
command line and prints its counts' checksum and the kernel used as JSON."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from analisi_gb300 import engine, workloads  # noqa: E402


def case():
    return workloads.small_case(88, 6000, 8, 40.0, 0.15, [3000, 2000, 1000], rmin=0.0, rmax=5.0,
                                nbin=50, tmax=3, skip=2, every=1, ntimesteps=4, primo=0)


if __name__ == "__main__":
    w = case()
    p = w["params"]
    with engine.Engine(0) as e:
        e.set_frames(w["positions"], w["boxes"], w["type_ids"], w["ntypes"])
        c = e.run(p["rmin"], p["rmax"], p["nbin"], p["tmax"], p["skip"], p["every"],
                  p["ntimesteps"], p["primo"], kernel=sys.argv[1])
        st = e.stats()
    print(json.dumps({"kernel_used": st["kernel_used"], "sum": int(c.sum()),
                      "weighted": int((c.astype(object) * (1 + __import__("numpy").arange(c.size)
                                                           .reshape(c.shape))).sum())}))
