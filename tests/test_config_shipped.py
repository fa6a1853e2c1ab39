"""config/main.conf parser on the reference's own shipped config files (config/*.conf and
scripts/**/*.conf): pg_conf_read_file must give every ConfigVal field exactly as the reference's
ConfigVal::read_file (read_config.h:122-297) gives it. The expected values are fixtures made by the
reference's own parser (tests/golden/make_conf_golden.py); the files themselves are read from the
reference checkout, so the test runs where that checkout is (and skips elsewhere). Where the
reference build is present the fixture is also re-derived live."""
import ctypes as C
import json
import os
import subprocess
import tempfile
import hashlib

import pytest

from perigrain_gb300 import _native as N

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.join(os.path.dirname(HERE), "oracle")
FIXTURE = os.path.join(HERE, "golden", "conf_shipped.json")


def _reference_root():
    r = subprocess.run(["make", "-s", "-C", ORACLE, "print-ref"], capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 else ""


REF = _reference_root()
with open(FIXTURE) as _f:
    SHIPPED = json.load(_f)
pytestmark = pytest.mark.skipif(not (REF and os.path.isdir(os.path.join(REF, "config"))),
                                reason="reference checkout (shipped config files) not present")


def ours(path):
    c = N.Conf()
    N.lib().pg_conf_default(C.byref(c))
    assert N.lib().pg_conf_read_file(C.byref(c), path.encode()) == 0
    return {k: getattr(c, k) for k, _ in N.Conf._fields_}


def test_fixture_covers_the_named_files():
    for rel in ("config/main.conf", "scripts/paper-collision/2d_collision_damping.conf",
                "scripts/3d_bulk_sphere/3d_bulk_sphere.conf"):
        assert rel in SHIPPED
    assert len(SHIPPED) >= 30


@pytest.mark.parametrize("rel", sorted(SHIPPED))
def test_shipped_config_parses_like_the_reference(rel):
    path = os.path.join(REF, rel)
    if not os.path.exists(path):
        pytest.skip("not in this checkout")
    with open(path, "rb") as f:
        assert hashlib.sha256(f.read()).hexdigest() == SHIPPED[rel]["sha256"], "file differs from the fixture's"
    want = SHIPPED[rel]["values"]
    got = ours(path)
    assert set(got) == set(want)
    for k, v in want.items():
        # every field exactly: integers and booleans as 0/1, doubles bit for bit
        assert got[k] == v, (rel, k, got[k], v)
    dump = os.path.join(ORACLE, "_ref", "conf_dump")
    if os.path.exists(dump):
        with tempfile.NamedTemporaryFile(suffix=".json") as t:
            subprocess.run([dump, path, t.name], check=True, capture_output=True)
            with open(t.name) as f:
                assert json.load(f) == want
