"""The -C writer's host dictionary codec (HostDictCodec, gsnp_gb300/csrc/
columns.cpp) against the codec's contract restated the plain way (sort,
unique, lower_bound; cpp/dict_compression.h:116-166), in
tests/native/dict_check.cpp.  The writer's files themselves are pinned by the
-C golden digests and the -C parity cases."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_host_dictionary_codec(tmp_path, native_lib):
    from gsnp_gb300 import build
    exe = str(tmp_path / "dict_check")
    csrc = os.path.join(ROOT, "gsnp_gb300", "csrc")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-pthread", "-I" + csrc,
                        "-I" + os.path.join(ROOT, "include"), "-I" + build._cuda_include(),
                        os.path.join(ROOT, "tests", "native", "dict_check.cpp"), os.path.join(csrc, "columns.cpp"),
                        "-o", exe, "-L" + build.LIBDIR, "-lgsnp_gb300", "-Wl,-rpath," + build.LIBDIR],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "checked" in r.stdout
