"""The -C files encoded on the GPU (columns_gpu.cu) equal, byte for byte,
those of the host encoder (columns.cpp), which the golden digests pin to the
reference's files.  The shapes cover windows of N only (c4's N block, longer
than a window), gap windows that show another window's counts (c4), deep
hotspots and copy-number segments (c2), known-SNP rows (c1, c5) and the
shorter last window of every chromosome."""
import os

import pytest

from gsnp_gb300 import api, synth

FILES = [".1_2", ".3_4_6", ".5_7_8_9_14_16", ".10", ".11_12_13", ".15_17"]


@pytest.mark.gpu
@pytest.mark.parametrize("name,scale", [("c0", 0.3), ("c1", 0.02), ("c2", 0.02), ("c4", 0.0101), ("c5", 0.01)])
def test_gpu_columns_equal_host_columns(name, scale, tmp_path, native_lib):
    w = synth.make_workload(name, scale=scale)
    flags = [f for f in w.cli_flags("dbsnp") if f != "-C"]
    c, _, _ = api.run_workload(w, flags, precision=api.PRECISION_FP32_FIXUP)
    try:
        out = {}
        for gpu in (1, 0):
            c.set_option("columns_gpu", gpu)
            base = str(tmp_path / ("gpu" if gpu else "host") / "cns")
            os.makedirs(os.path.dirname(base))
            rc = c.lib.gsnp_write_columns(c.ctx, w.chr_name.encode(), base.encode())
            assert rc == 0, c.lib.gsnp_context_error(c.ctx)
            out[gpu] = {f: open(base + f, "rb").read() for f in FILES}
    finally:
        c.close()
    for f in FILES:
        assert out[1][f] == out[0][f], f"{name}: {f} differs between the GPU and host encoders"
