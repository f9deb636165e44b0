"""HDF5 subset (phantom / result files) and the `spinwalk sim -c cfg.ini` drop-in path."""
import glob
import os
import shutil
import subprocess

import numpy as np
import pytest

from spinwalk_gb300 import _lib
from spinwalk_gb300.problem import Problem, cylinder_phantom
from tests import oracle_lib
from tests.helpers import ROOT, bits_equal, m_close


def test_h5_roundtrip(tmp_path):
    rng = np.random.default_rng(0)
    data = {"mask": rng.integers(0, 3, (5, 6, 7), dtype=np.uint8),
            "fieldmap": rng.normal(size=(5, 6, 7)).astype(np.float32),
            "fov": np.array([1e-4, 2e-4, 3e-4], np.float32),
            "zz_double": rng.normal(size=(4, 2)),
            "empty": np.zeros((0, 3), np.float32)}
    f = tmp_path / "p.h5"
    _lib.h5_write(f, data)
    assert f.read_bytes()[:8] == b"\x89HDF\r\n\x1a\n"
    for k, v in data.items():
        got = _lib.h5_read(f, k)
        assert got.dtype == v.dtype and got.shape == v.shape
        assert bits_equal(got, v), k
    with pytest.raises(_lib.SpinWalkError):
        _lib.h5_read(f, "missing")


def test_h5_integer_types_roundtrip(tmp_path):
    """Integer datasets of every width and signedness (MATLAB writes masks as int8, h5py may
    write int64): stored and read back with their own type."""
    rng = np.random.default_rng(1)
    data = {f"d_{np.dtype(t).name}": rng.integers(np.iinfo(t).min, np.iinfo(t).max, (3, 4, 5),
                                                  dtype=t, endpoint=True)
            for t in (np.int8, np.uint16, np.int16, np.uint32, np.int32, np.uint64, np.int64)}
    f = tmp_path / "ints.h5"
    _lib.h5_write(f, data)
    for k, v in data.items():
        got = _lib.h5_read(f, k)
        assert got.dtype == v.dtype and bits_equal(got, v), k


def test_h5_type_conversion_rules(tmp_path):
    """The conversion sw_run_config applies to datasets stored in other types than the
    reference reads (mask uint8, the rest float), with libhdf5's rules (tests/h5_convert_check.cpp)."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "h5_convert_check"
    csrc = os.path.join(ROOT, "spinwalk_gb300", "csrc")
    subprocess.run([gxx, "-O2", "-std=c++17", f"-I{csrc}",
                    os.path.join(ROOT, "tests", "h5_convert_check.cpp"), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout


def test_h5_reads_a_libhdf5_file():
    """A file written by libhdf5 itself (a MATLAB v7.3 test file shipped with scipy: HDF5 behind
    a 512-byte user block, version-1 layout messages)."""
    scipy = pytest.importorskip("scipy")
    hits = glob.glob(os.path.join(os.path.dirname(scipy.__file__), "io", "matlab", "tests", "data",
                                  "testhdf5_7.4_GLNX86.mat"))
    if not hits:
        pytest.skip("scipy test data not installed")
    got = _lib.h5_read(hits[0], "testdouble")
    assert got.shape == (9, 1)
    assert np.allclose(got.ravel(), np.arange(9) * np.pi / 4)


GRAD_T = (200, 400, 600, 800, 1600, 1800, 2000, 2200)
GRAD_X = (30.0, 30.0, 30.0, 0.0, 30.0, 30.0, 30.0, 0.0)


def _write_case(tmp, scale_type, scales):
    mask, field = cylinder_phantom(20, 20e-6, 3e-6, 0.1, seed=3)
    _lib.h5_write(tmp / "phantom.h5", {"mask": mask, "fieldmap": field,
                                       "fov": np.array([20e-6] * 3, np.float32)})
    scale_lines = "\n".join(f"SCALE[{i}] = {s}" for i, s in enumerate(scales))
    (tmp / "cfg.ini").write_text(f"""
[GENERAL]
SEQ_NAME = test
[FILES]
OUTPUT_DIR = out
PHANTOM[0] = phantom.h5
[TISSUE_PARAMETERS]
DIFFUSIVITY[0] = 1e-9
DIFFUSIVITY[1] = 1e-9
P_XY[0] = 1 0.2
P_XY[1] = 0.3 1
T1[0] = 2000
T1[1] = 2000
T2[0] = 40
T2[1] = 20
[SCAN_PARAMETERS]
TR = 3050
TE = 1000 3000
RF_FA = 90 180
RF_PH = 0 90
RF_T = 0 1500
TIME_STEP = 50
DUMMY_SCAN = 1
LINEAR_PHASE_CYCLING = 10
GRADIENT_T = {" ".join(str(t) for t in GRAD_T)}
GRADIENT_X = {" ".join(str(g) for g in GRAD_X)}
GRADIENT_Y = {" ".join("0" for _ in GRAD_T)}
GRADIENT_Z = {" ".join("0" for _ in GRAD_T)}
[SIMULATION_PARAMETERS]
B0 = 9.4
SEED = 10
NUMBER_OF_SPINS = 300
CROSS_FOV = 1
WHAT_TO_SCALE = {scale_type}
{scale_lines}
""")
    return mask, field


@pytest.mark.gpu
@pytest.mark.parametrize("scale_type,scales", [(0, [1.0, 0.5, 2.0]), (2, [0.0, 1.0, 3.0]),
                                              (1, [0.0, 0.5, 2.0, 3.0]), (1, [1.0, 1.0])])
def test_run_config_matches_oracle_per_scale(tmp_path, scale_type, scales):
    mask, field = _write_case(tmp_path, scale_type, scales)
    r = subprocess.run([os.path.join(ROOT, "spinwalk_gb300", "spinwalk"), "-l",
                        str(tmp_path / "run.log"), "sim", "-c", str(tmp_path / "cfg.ini")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "Finished " + str(tmp_path / "cfg.ini") in (tmp_path / "run.log").read_text()
    out = tmp_path / "out" / "test_phantom.h5"
    M, XYZ, T = _lib.h5_read(out, "M"), _lib.h5_read(out, "XYZ"), _lib.h5_read(out, "T")
    assert M.shape == (len(scales), 300, 2, 3) and T.shape == (len(scales), 300, 2, 1)
    assert np.allclose(_lib.h5_read(out, "scales").ravel(), scales)
    assert np.allclose(_lib.h5_read(out, "TE").ravel(), [1e-3, 3e-3])
    xyz0 = _lib.initial_positions([20e-6] * 3, 10, 300)
    for k, s in enumerate(scales):
        s32 = np.float32(s)
        g = np.zeros((len(GRAD_T), 3), np.float32)
        g[:, 0] = np.asarray(GRAD_X, np.float32) * (s32 if scale_type == 1 else np.float32(1))
        kw = dict(TR_us=3050, TE_us=(1000, 3000), RF_FA=(90.0, 180.0), RF_PH=(0.0, 90.0),
                  RF_us=(0, 1500), pXY=[[1, 0.2], [0.3, 1]], n_dummy_scan=1, n_spins=300, seed=10,
                  diffusivity=(float(np.float32(1e-9)),) * 2,      # the INI value is std::stof'd
                  gradient_us=GRAD_T, gradient_xyz=g)
        if scale_type == 0:
            fov = [float(s32 * np.float32(20e-6))] * 3
            pr = Problem(mask, fov, field, XYZ0=(xyz0 * s32).astype(np.float32),
                         linear_phase_cycling=10.0, **kw)
            pr.params.fov[:] = [float(s32 * np.float32(20e-6))] * 3
        elif scale_type == 1:
            pr = Problem(mask, [20e-6] * 3, field, XYZ0=xyz0, linear_phase_cycling=10.0, **kw)
        else:
            pr = Problem(mask, [20e-6] * 3, field, XYZ0=xyz0,
                         linear_phase_cycling=float(np.float32(10.0) * s32), **kw)
        o = oracle_lib.run(pr)
        assert bits_equal(XYZ[k], o["XYZ1"]), k
        assert bits_equal(T[k][..., 0], o["T"]), k
        ok, rel = m_close(M[k], o["M1"])
        assert ok, (k, rel)


def test_cli_rejects_cpu_flag_and_bad_config(tmp_path):
    exe = os.path.join(ROOT, "spinwalk_gb300", "spinwalk")
    r = subprocess.run([exe, "sim", "-c", "x.ini", "-p"], capture_output=True, text=True,
                       cwd=tmp_path)
    assert r.returncode == 1 and "GPU only" in r.stderr
    assert "GPU only" in (tmp_path / "log_spinwalk.txt").read_text()
    (tmp_path / "bad.ini").write_text("[SCAN_PARAMETERS]\nTE = 5 1\n")
    assert _lib.config_dump(str(tmp_path / "bad.ini"), tmp_path / "d.txt") != 0


def test_cli_log_file_and_option_forms(tmp_path):
    """The reference's global -l/--log option (default log_spinwalk.txt in the working
    directory, appended): the CLI accepts it in both forms, and a failed config is logged."""
    exe = os.path.join(ROOT, "spinwalk_gb300", "spinwalk")
    missing = str(tmp_path / "missing.ini")
    for args, log in ((["-l", str(tmp_path / "a.log"), "sim", "-c", missing], tmp_path / "a.log"),
                      ([f"--log={tmp_path / 'b.log'}", "sim", f"--configs={missing}", "--device=0"],
                       tmp_path / "b.log"),
                      (["sim", "-c", missing, "-d", "0"], tmp_path / "log_spinwalk.txt")):
        r = subprocess.run([exe, *args], capture_output=True, text=True, cwd=tmp_path)
        assert r.returncode == 1, r.stdout + r.stderr
        assert "Aborting" in r.stdout
        lines = log.read_text().splitlines()
        assert any("[info]: Simulating " + missing in ln for ln in lines)
        err = [ln for ln in lines if "[error]: " + missing + ": " in ln]
        assert err and all(ln.split(missing + ": ", 1)[1].strip() for ln in err), lines
    r = subprocess.run([exe, "--log"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 1 and "usage" in r.stderr


def test_driver_errors_set_last_error(tmp_path):
    """Errors of the HDF5 helpers and of the driver come back as a code plus a message in
    sw_last_error(), like every other entry point."""
    with pytest.raises(_lib.SpinWalkError, match=r"spinwalk error -?\d+: \S"):
        _lib.h5_read(tmp_path / "none.h5", "M")
    _lib.h5_write(tmp_path / "ok.h5", {"M": np.zeros((2, 3), np.float32)})
    with pytest.raises(_lib.SpinWalkError, match=r"spinwalk error -?\d+: \S"):
        _lib.h5_read(tmp_path / "ok.h5", "no_such_dataset")
    with pytest.raises(_lib.SpinWalkError, match=r"spinwalk error -?\d+: \S"):
        _lib.run_config(tmp_path / "missing.ini")


@pytest.mark.gpu
def test_run_config_reads_matlab_style_phantom(tmp_path):
    """The reference README's MATLAB recipe stores the mask as int8 (MATLAB has no uint8 HDF5
    writer) and h5py users often keep float64 arrays: the same config run on such a phantom
    (int8 mask, float64 fieldmap and fov, float32 values widened) writes the result file of the
    uint8 / float32 phantom, bit for bit."""
    mask, field = _write_case(tmp_path, 0, [1.0, 2.0])
    _lib.h5_write(tmp_path / "phantom_m.h5", {"mask": mask.astype(np.int8),
                                              "fieldmap": field.astype(np.float64),
                                              "fov": np.array([20e-6] * 3, np.float32).astype(np.float64)})
    cfg = (tmp_path / "cfg.ini").read_text()
    (tmp_path / "cfg_m.ini").write_text(cfg.replace("PHANTOM[0] = phantom.h5", "PHANTOM[0] = phantom_m.h5"))
    exe = os.path.join(ROOT, "spinwalk_gb300", "spinwalk")
    for ini in ("cfg.ini", "cfg_m.ini"):
        r = subprocess.run([exe, "-l", str(tmp_path / "run.log"), "sim", "-c", str(tmp_path / ini)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    a, b = tmp_path / "out" / "test_phantom.h5", tmp_path / "out" / "test_phantom_m.h5"
    for k in ("M", "XYZ", "T", "scales", "TE"):
        assert bits_equal(_lib.h5_read(a, k), _lib.h5_read(b, k)), k


def _expect_run_error(ini, *fragments):
    with pytest.raises(_lib.SpinWalkError) as e:
        _lib.run_config(ini)
    for f in fragments:
        assert f in str(e.value), str(e.value)


def test_run_config_input_checks(tmp_path):
    """Phantom and start-file checks of sw_run_config, made before any GPU is selected: fov,
    XYZ and M must have exactly the size the reference reads them with (h5_helper::read without
    resizing fails on any other size); a fieldmap must have as many voxels as the mask (the
    reference would read past a shorter one)."""
    mask, field = _write_case(tmp_path, 0, [1.0])
    cfg = (tmp_path / "cfg.ini").read_text()
    fov = np.array([20e-6] * 3, np.float32)

    def case(name, phantom=None, xyz=None, m=None):
        d = tmp_path / name
        d.mkdir()
        _lib.h5_write(d / "phantom.h5", phantom or {"mask": mask, "fieldmap": field, "fov": fov})
        extra = ""
        if xyz is not None:
            _lib.h5_write(d / "xyz.h5", {"XYZ": xyz})
            extra += "XYZ0[0] = xyz.h5\n"
        if m is not None:
            _lib.h5_write(d / "m.h5", {"M": m})
            extra += "M0[0] = m.h5\n"
        (d / "cfg.ini").write_text(cfg.replace("PHANTOM[0] = phantom.h5",
                                               "PHANTOM[0] = phantom.h5\n" + extra))
        return d / "cfg.ini"

    _expect_run_error(case("fov4", {"mask": mask, "fov": np.append(fov, 1e-6).astype(np.float32)}),
                      '"fov" has different size 4 vs 3')
    _expect_run_error(case("short_field", {"mask": mask, "fieldmap": field.ravel()[:-1].copy(),
                                           "fov": fov}), "fieldmap has", "voxels")
    xyz = np.full((301, 3), 10e-6, np.float32)
    _expect_run_error(case("xyz_long", xyz=xyz), '"XYZ" has different size 903 vs 900')
    _expect_run_error(case("xyz_out", xyz=np.full((300, 3), 30e-6, np.float32)),
                      "outside the FoV")
    _expect_run_error(case("m_short", xyz=xyz[:300].copy(), m=np.zeros((299, 3), np.float32)),
                      '"M" has different size 897 vs 900')
    # valid inputs get as far as selecting the device (none on a CPU-only machine)
    if _lib.device_count() == 0:
        _expect_run_error(case("valid", xyz=xyz[:300].copy(), m=np.zeros((300, 3), np.float32)),
                          "device 0 is not available")


@pytest.mark.parametrize("dtype", [np.uint8, np.int8, np.int16, np.float32, np.float64])
@pytest.mark.parametrize("filters,level,version", [
    (("shuffle", "deflate"), 6, 1), (("deflate",), 9, 2), (("deflate",), 1, 1),
    (("deflate",), 0, 2), (("shuffle",), 6, 1), ((), 6, 1), (("shuffle", "deflate", "fletcher32"), 4, 2)])
def test_h5_chunked_datasets(tmp_path, dtype, filters, level, version):
    """Chunked datasets (h5py's compression="gzip", MATLAB's compressed files): partial edge
    chunks, deflate streams from zlib at several levels (stored, fixed and dynamic Huffman
    blocks), shuffle and fletcher32, filter pipeline messages of versions 1 and 2."""
    from tests.h5_chunked import write_chunked
    rng = np.random.default_rng(int(level) + len(filters))
    shape = (13, 17, 9)
    if np.dtype(dtype).kind == "f":
        a = rng.normal(size=shape).astype(dtype)
        a[:4] = np.round(a[:4])                    # some compressible rows
    else:
        info = np.iinfo(dtype)
        a = rng.integers(info.min, info.max, shape, dtype=dtype, endpoint=True)
        a[5:] //= 16                               # long runs of small values
    f = tmp_path / "c.h5"
    write_chunked(f, "fieldmap", a, (4, 5, 3), filters=filters, level=level,
                  pipeline_version=version)
    got = _lib.h5_read(f, "fieldmap")
    assert got.dtype == a.dtype and got.shape == a.shape
    assert bits_equal(got, a)


def test_h5_chunked_index_shapes(tmp_path):
    """Two-level chunk B-trees, unwritten chunks (zeros), chunks stored with every filter
    skipped, ranks 1 and 4, a compressible phantom-like mask."""
    from tests.h5_chunked import write_chunked
    rng = np.random.default_rng(5)
    mask = (rng.random((40, 40, 40)) < 0.05).astype(np.uint8)
    write_chunked(tmp_path / "m.h5", "mask", mask, (8, 8, 8), leaf_entries=7)
    assert bits_equal(_lib.h5_read(tmp_path / "m.h5", "mask"), mask)
    a = rng.normal(size=(6, 7, 8)).astype(np.float32)
    write_chunked(tmp_path / "s.h5", "x", a, (2, 4, 8), skip_chunks={(0, 1, 0), (2, 0, 0)},
                  raw_chunks={(1, 1, 0)}, leaf_entries=2)
    want = a.copy()
    want[0:2, 4:7, :] = 0
    want[4:6, 0:4, :] = 0
    assert bits_equal(_lib.h5_read(tmp_path / "s.h5", "x"), want)
    v = rng.normal(size=(1000,))
    write_chunked(tmp_path / "v.h5", "v", v, (64,))
    assert bits_equal(_lib.h5_read(tmp_path / "v.h5", "v"), v)
    w = rng.integers(0, 100, (3, 4, 5, 6), dtype=np.int32)
    write_chunked(tmp_path / "w.h5", "w", w, (2, 3, 2, 4), leaf_entries=5)
    assert bits_equal(_lib.h5_read(tmp_path / "w.h5", "w"), w)
    z = np.zeros((5, 5, 5), np.float32)
    write_chunked(tmp_path / "z.h5", "z", np.ones((5, 5, 5), np.float32), (5, 5, 5),
                  skip_chunks={(0, 0, 0)})
    assert bits_equal(_lib.h5_read(tmp_path / "z.h5", "z"), z)


def test_h5_chunked_errors(tmp_path):
    """A corrupted deflate stream and an unsupported filter are errors naming the dataset,
    never data."""
    import struct
    from tests.h5_chunked import write_chunked
    a = np.arange(4000, dtype=np.float32).reshape(10, 20, 20)
    f = tmp_path / "c.h5"
    write_chunked(f, "fieldmap", a, (5, 20, 20), filters=("deflate",))
    b = bytearray(f.read_bytes())
    at = b.find(bytes([0x78, 0x9C]))               # first zlib stream (level 6 header)
    assert at > 0
    b[at + 40] ^= 0xFF
    f.write_bytes(bytes(b))
    with pytest.raises(_lib.SpinWalkError, match="fieldmap: .*deflate"):
        _lib.h5_read(f, "fieldmap")
    write_chunked(f, "fieldmap", a, (5, 20, 20), filters=("deflate",))
    b = bytearray(f.read_bytes())
    at = b.find(b"deflate\0")                     # the filter's name in a version-1 pipeline
    assert at > 8 and struct.unpack_from("<H", b, at - 8)[0] == 1
    struct.pack_into("<H", b, at - 8, 32000)       # its id -> LZF
    f.write_bytes(bytes(b))
    with pytest.raises(_lib.SpinWalkError, match="fieldmap: unsupported HDF5 filter 32000"):
        _lib.h5_read(f, "fieldmap")


def test_h5_deflate_streams_of_every_zlib_strategy(tmp_path):
    """The deflate decoder on streams of every zlib strategy (default, filtered, Huffman only,
    run-length, fixed codes), levels 0-9 and windows 2^9-2^15, over random, sparse, run-length,
    periodic and smooth data in chunks of 1 byte up to the whole array."""
    import zlib
    from tests.h5_chunked import write_chunked
    rng = np.random.default_rng(11)
    strategies = [zlib.Z_DEFAULT_STRATEGY, zlib.Z_FILTERED, zlib.Z_HUFFMAN_ONLY, zlib.Z_RLE,
                  zlib.Z_FIXED]
    for trial in range(80):
        size = int(rng.integers(1, 40000))
        kind = trial % 5
        if kind == 0:
            a = rng.integers(0, 256, size, dtype=np.uint8)
        elif kind == 1:
            a = (rng.random(size) < 0.02).astype(np.uint8)
        elif kind == 2:
            a = np.repeat(rng.integers(0, 4, size // 37 + 1, dtype=np.uint8), 37)[:size]
        elif kind == 3:
            a = (np.arange(size) % int(rng.integers(1, 300))).astype(np.uint8)
        else:
            s = np.sin(np.arange(size // 4 + 1) * 1e-3).astype(np.float32)
            a = np.frombuffer(s.tobytes(), np.uint8)[:size].copy()
        f = tmp_path / "x.h5"
        write_chunked(f, "x", a, (int(rng.integers(1, size + 1)),), filters=("deflate",),
                      level=int(rng.integers(0, 10)), strategy=strategies[trial % 5],
                      wbits=int(rng.integers(9, 16)), leaf_entries=16)
        assert bits_equal(_lib.h5_read(f, "x"), a), trial


def test_h5_damaged_files_are_errors(tmp_path):
    """Damaged phantom files (random bytes, bit flips, truncations, huge 8-byte size fields) in
    contiguous and chunked layouts either read or fail with an error: no crash, no huge
    allocation (a size the file cannot hold is refused)."""
    from tests.h5_chunked import write_chunked
    rng = np.random.default_rng(17)
    _lib.h5_write(tmp_path / "a.h5", {"x": rng.normal(size=(7, 8, 9)).astype(np.float32),
                                      "mask": np.zeros((4, 4, 4), np.uint8)})
    write_chunked(tmp_path / "b.h5", "x", rng.normal(size=(20, 20, 20)), (5, 7, 20),
                  filters=("shuffle", "deflate", "fletcher32"), leaf_entries=3)
    outcomes = {"read": 0, "error": 0}
    for src in ("a.h5", "b.h5"):
        raw = (tmp_path / src).read_bytes()
        for k in range(150):
            c = bytearray(raw)
            mode = k % 4
            if mode == 0:
                for _ in range(int(rng.integers(1, 4))):
                    c[int(rng.integers(0, len(c)))] = int(rng.integers(0, 256))
            elif mode == 1:
                c = c[:int(rng.integers(0, len(c)))]
            elif mode == 2:
                i = int(rng.integers(0, len(c) - 8))
                c[i:i + 8] = int(rng.integers(0, 2 ** 63)).to_bytes(8, "little")
            else:
                c[int(rng.integers(0, len(c)))] ^= 1 << int(rng.integers(0, 8))
            f = tmp_path / "d.h5"
            f.write_bytes(bytes(c))
            try:
                _lib.h5_read(f, "x")
                outcomes["read"] += 1
            except _lib.SpinWalkError:
                outcomes["error"] += 1
    assert outcomes["error"] > 100 and sum(outcomes.values()) == 300


def test_h5_reads_only_what_it_needs(tmp_path):
    """Files are memory-mapped: reading the 3 values of `fov` from a 165 MB phantom does not load
    the phantom (the first reader copied the whole file per read, ~0.7 s here), and the large
    datasets come back intact."""
    import time
    n = 320
    rng = np.random.default_rng(2)
    field = np.zeros((n, n, n), np.float32)
    field[::7, ::5, ::3] = rng.normal(size=field[::7, ::5, ::3].shape)
    mask = (field > 1).astype(np.uint8)
    fov = np.array([3.2e-4] * 3, np.float32)
    f = tmp_path / "big.h5"
    _lib.h5_write(f, {"mask": mask, "fieldmap": field, "fov": fov})
    t = time.perf_counter()
    for _ in range(10):
        got = _lib.h5_read(f, "fov")
    assert (time.perf_counter() - t) / 10 < 0.05
    assert bits_equal(got, fov)
    assert bits_equal(_lib.h5_read(f, "mask"), mask)
    assert bits_equal(_lib.h5_read(f, "fieldmap"), field)
