import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def reference_tree():
    """The reference source tree the reference programs were built from
    (GB_REFERENCE, else the record the build leaves beside them), or None
    where it is absent (the GPU machine)."""
    env = os.environ.get("GB_REFERENCE")
    rec = ROOT / "oracle" / "_ref" / "REFERENCE_TREE"
    p = Path(env) if env else (Path(rec.read_text().strip()) if rec.exists() else None)
    return p if p is not None and p.exists() else None


def golden(name: str):
    return np.load(GOLDEN / name, allow_pickle=False)


@pytest.fixture(scope="session")
def scene_dir(tmp_path_factory):
    """Scene text files of the seeded workloads (octrees are built by the
    library's builder, identical to the reference oconv's)."""
    from pyradiance_gb300 import workloads as w
    d = tmp_path_factory.mktemp("scenes")
    for name, text in (("c1", w.daylight_room()), ("c2", w.window_room()), ("zoo", w.shape_zoo()),
                       ("c2e", w.window_room(ntri=0)), ("glossy", w.glossy_room())):
        (d / f"{name}.rad").write_text(text)
    return d


MODS_C2 = [dict(modifier="groundglow"),
           dict(modifier="skyglow", calfile="reinhartb.cal", params="MF=1", binv="rbin", nbins="Nrbins")]


def zscores(mean_a, se_a, mean_b, se_b):
    se = np.sqrt(se_a ** 2 + se_b ** 2)
    m = se > 0
    return (mean_a - mean_b)[m] / se[m]

# bin groups of the 146 rcontrib columns: ground, then the 8 Reinhart MF:1 rows
ROW_EDGES = [0, 1, 31, 61, 85, 109, 127, 139, 145, 146]
