"""The library's INI reader against the reference's config_reader (src/sim/config_reader.cpp,
built from its sources into oracle/_ref): both parse the same files into the same parameters."""
import os

import pytest

from spinwalk_gb300 import _lib
from tests import oracle_lib

PARENT = """
; parent config: defaults
[GENERAL]
PARENT_CONFIG =
SEQ_NAME      = parent_seq

[FILES]
OUTPUT_DIR   = out_dir
PHANTOM[0]  = ph_a.h5
PHANTOM[1]  = sub/ph_b.h5
XYZ0[0]   =
M0[0]   =

[TISSUE_PARAMETERS]
DIFFUSIVITY[0] = 1.0e-9
DIFFUSIVITY[1] = 2.5e-9
P_XY[0] = 1.0 0.3
P_XY[1] = 0.2 1.0
T1[0] = 2200
T1[1] = 1500.5
T2[0] = 41
T2[1] = 20

[SCAN_PARAMETERS]
TR = 10e3
TE = 5e3 6e3 7e3
RF_FA = 15.0 0.0 0.0
RF_PH = 0.0 0.0 0.0
RF_T = 0 100e3 200e3
DEPHASING =
DEPHASING_T =
GRADIENT_X =
GRADIENT_Y =
GRADIENT_Z =
GRADIENT_T =
TIME_STEP  = 50
DUMMY_SCAN  = 0
LINEAR_PHASE_CYCLING = 0
QUADRATIC_PHASE_CYCLING = 0

[SIMULATION_PARAMETERS]
B0   = 9.4
SEED = 0
NUMBER_OF_SPINS = 1e5
CROSS_FOV = 0
RECORD_TRAJECTORY = 0
MAX_ITERATIONS = 1e4
WHAT_TO_SCALE = 0
SCALE[0] = 0.0125
SCALE[1] = 0.0147
SCALE[2] = 1.9803
"""

CHILDREN = {
    "gre": """
[GENERAL]
PARENT_CONFIG = parent.ini
SEQ_NAME     = gre
[SCAN_PARAMETERS]
TR = 40000
TE = 20000
RF_FA = 90.0
RF_PH = 0.0
RF_T = 0
[SIMULATION_PARAMETERS]
SEED = 10
""",
    "se_gradients": """
[GENERAL]
PARENT_CONFIG = parent.ini
SEQ_NAME = se
[FILES]
PHANTOM[0] = ph_a.h5
[SCAN_PARAMETERS]
TR = 40e3
TE = 20000   ; trailing text after a value
RF_FA = 90.0 180.0
RF_PH = 0.0 90
RF_T = 0 10000
GRADIENT_X = 0 521.9377 0
GRADIENT_Y = 0 0 0
GRADIENT_Z = 1.5e1 0 -3
GRADIENT_T = 950 1000 3000
DEPHASING = 360 720
DEPHASING_T = 10e3 30e3
TIME_STEP = 25
DUMMY_SCAN = -1
LINEAR_PHASE_CYCLING = 5.625
[SIMULATION_PARAMETERS]
SEED = 7
NUMBER_OF_SPINS = 2.5e4
CROSS_FOV = 1
RECORD_TRAJECTORY = 1
WHAT_TO_SCALE = 2
SCALE[0] = 0
SCALE[1] = 1
SCALE[2] = 2
B0 = 7
""",
    "tissue_override": """
[GENERAL]
PARENT_CONFIG = parent.ini
[TISSUE_PARAMETERS]
DIFFUSIVITY[0] = 3e-9
T1[0] = 1000
T2[0] = 30
P_XY[0] = 1
[SCAN_PARAMETERS]
TE = 5000
RF_FA = 30
RF_PH = 0
RF_T = 0
""",
    "bad_rf_sizes": """
[GENERAL]
PARENT_CONFIG = parent.ini
[SCAN_PARAMETERS]
RF_FA = 90 180
RF_T = 0
""",
    "bad_te_order": """
[GENERAL]
PARENT_CONFIG = parent.ini
[SCAN_PARAMETERS]
TE = 7000 5000
""",
    "missing_file": """
[GENERAL]
PARENT_CONFIG = parent.ini
[FILES]
PHANTOM[0] = does_not_exist.h5
""",
}


@pytest.fixture()
def cfgdir(tmp_path):
    (tmp_path / "sub").mkdir()
    for f in ("ph_a.h5", "sub/ph_b.h5"):
        (tmp_path / f).write_bytes(b"")
    (tmp_path / "parent.ini").write_text(PARENT)
    for name, text in CHILDREN.items():
        (tmp_path / f"{name}.ini").write_text(text)
    return tmp_path


@pytest.mark.skipif(not oracle_lib.ref_available(), reason="reference source tree not present")
@pytest.mark.parametrize("name", ["parent"] + list(CHILDREN))
def test_config_reader_matches_reference(cfgdir, name):
    ini = str(cfgdir / f"{name}.ini")
    ours, ref = cfgdir / f"{name}.ours.txt", cfgdir / f"{name}.ref.txt"
    rc = _lib.config_dump(ini, ours)
    ok_ref = oracle_lib.ref().ref_config_dump(ini.encode(), str(ref).encode())
    assert (rc == 0) == (ok_ref == 1)
    assert ours.read_text() == ref.read_text()


def test_config_reader_semantics(cfgdir):
    """Pinned values (no reference needed): parent inheritance, float-parsed vectors,
    microseconds -> time points, relative paths."""
    out = cfgdir / "se.txt"
    assert _lib.config_dump(str(cfgdir / "se_gradients.ini"), out) == 0
    d = {}
    for line in out.read_text().splitlines():
        parts = line.split()
        if parts and not line.startswith("  "):
            d[parts[0]] = parts[1:]
    assert d["TR_us"] == ["40000"] and d["timestep_us"] == ["25"]
    assert d["TE_us"] == ["800"]                       # 20000 us / 25 us
    assert d["gradient_us"] == ["38", "40", "120"]
    assert d["n_dummy_scan"] == ["-1"]                 # prepare() resolves it later
    assert d["scale_type"] == ["2"] and d["scales"] == ["0", "1", "2"]
    assert d["n_spins"] == ["25000"] and d["seed"] == ["7"]
    assert d["diffusivity"][0] == "9.9999997171806854e-10"   # std::stof then widened
    assert os.path.isabs(d["output"][0]) and d["output"][0].endswith("se_ph_a.h5")
    assert _lib.config_dump(str(cfgdir / "bad_te_order.ini"), cfgdir / "x.txt") != 0


def _ref_config_dir():
    from spinwalk_gb300 import _build
    return os.path.join(_build.REF_TREE, "config")


REF_CONFIG_DIR = _ref_config_dir()


@pytest.mark.skipif(not (oracle_lib.ref_available() and os.path.isdir(REF_CONFIG_DIR)),
                    reason="reference source tree not present")
def test_config_reader_matches_reference_on_its_shipped_configs(tmp_path):
    """Every config file the reference ships (config/*.ini: default, GRE, SE, bSSFP, GRASE,
    stimulated echo, gradients), parsed by both readers into the same parameters. They are
    copied two levels down in a scratch tree, with empty files where they name phantoms and
    start files (../../phantoms/...), so that both readers get past their file checks."""
    import re
    import shutil
    cfg = tmp_path / "a" / "b"
    cfg.mkdir(parents=True)
    names = sorted(f for f in os.listdir(REF_CONFIG_DIR) if f.endswith(".ini"))
    assert len(names) >= 7
    for f in names:
        text = open(os.path.join(REF_CONFIG_DIR, f)).read()
        shutil.copy(os.path.join(REF_CONFIG_DIR, f), cfg / f)
        for m in re.finditer(r"^\s*(?:PHANTOM|XYZ0|M0)\[\d+\]\s*=\s*(\S+)", text, re.M):
            p = (cfg / m.group(1)).resolve()
            p.parent.mkdir(parents=True, exist_ok=True)
            p.touch()
    parsed = []
    for f in names:
        ours, ref = tmp_path / f"{f}.ours.txt", tmp_path / f"{f}.ref.txt"
        rc = _lib.config_dump(str(cfg / f), ours)
        ok_ref = oracle_lib.ref().ref_config_dump(str(cfg / f).encode(), str(ref).encode())
        assert (rc == 0) == (ok_ref == 1), f
        if rc == 0:
            assert ours.read_text() == ref.read_text(), f
            parsed.append(f)
    assert len(parsed) >= 6, parsed


def test_config_parent_cycle_is_an_error(tmp_path):
    """A config that is its own ancestor through PARENT_CONFIG (directly or via another file)
    is refused with a message; the reference's reader would recurse until the stack overflows."""
    from spinwalk_gb300 import _lib as L
    (tmp_path / "self.ini").write_text("[GENERAL]\nPARENT_CONFIG = self.ini\nSEQ_NAME = s\n")
    (tmp_path / "a.ini").write_text("[GENERAL]\nPARENT_CONFIG = sub/../b.ini\n")
    (tmp_path / "sub").mkdir()
    (tmp_path / "b.ini").write_text("[GENERAL]\nPARENT_CONFIG = a.ini\n")
    for name in ("self.ini", "a.ini"):
        assert L.config_dump(str(tmp_path / name), tmp_path / "out.txt") != 0
        assert b"PARENT_CONFIG cycle" in L.lib().sw_last_error()
