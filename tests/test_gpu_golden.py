"""GPU engine against the reference-generated fixtures: counts per reference
thread partition (nparts = the reference's nthreads) folded by
gofr_counts_to_buffer reproduce the reference's double result buffer bit for
bit, with both the FP32+recheck kernel and the plain FP64 kernel."""
import numpy as np
import pytest

import golden_util as gu

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel", ["auto", "f64"])
@pytest.mark.parametrize("name", gu.names())
def test_gpu_reproduces_reference_buffer(gpu_engine, name, kernel):
    from analisi_gb300 import engine
    g = gu.load(name)
    m = g["meta"]
    gpu_engine.set_frames(g["internal_positions"], g["internal_boxes"], g["internal_type_ids"],
                          m["ntypes"], triclinic=m["triclinic"])
    nparts = max(1, m["nthreads"])
    c = gpu_engine.run(m["rmin"], m["rmax"], m["nbin"], m["tmax"], m["skip"], m["every"],
                       m["ntimesteps"], m["primo"], kernel=kernel, nparts=nparts)
    if nparts == 1:
        c = c[None]
    buf = engine.counts_to_buffer(c, m["ntimesteps"], m["skip"], nparts=nparts)
    ref = g["ref_buffer"]
    assert np.array_equal(np.rint(ref / gu.incr(m)).astype(np.uint64), c.sum(axis=0))
    assert np.array_equal(buf.view(np.uint64), ref.view(np.uint64))
