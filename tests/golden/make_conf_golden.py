"""Generate tests/golden/conf_shipped.json: every config file the reference ships (config/*.conf
and scripts/**/*.conf), parsed by the reference's own ConfigVal::read_file (read_config.h:122-297)
through oracle/_ref/conf_dump (the reference header compiled unmodified by oracle/Makefile).

Stores, per file (path relative to the reference checkout), the SHA-256 of its bytes and every
ConfigVal field. Needs the reference checkout that oracle/Makefile reads. Run from the repository
root:
    python tests/golden/make_conf_golden.py
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
ORACLE = os.path.join(ROOT, "oracle")


def reference_root():
    return subprocess.run(["make", "-s", "-C", ORACLE, "print-ref"], check=True, capture_output=True,
                          text=True).stdout.strip()


def shipped_confs(ref):
    out = []
    for top in ("config", "scripts"):
        for d, _, files in os.walk(os.path.join(ref, top)):
            out += [os.path.relpath(os.path.join(d, f), ref) for f in files if f.endswith(".conf")]
    return sorted(out)


def reference_parse(path):
    exe = os.path.join(ORACLE, "_ref", "conf_dump")
    with tempfile.NamedTemporaryFile(suffix=".json") as t:
        subprocess.run([exe, path, t.name], check=True, capture_output=True)
        with open(t.name) as f:
            return json.load(f)


def main():
    subprocess.run(["make", "-s", "-C", ORACLE], check=True)
    ref = reference_root()
    if not os.path.exists(os.path.join(ORACLE, "_ref", "conf_dump")):
        sys.exit("reference build unavailable (oracle/_ref/conf_dump)")
    fixture = {}
    for rel in shipped_confs(ref):
        p = os.path.join(ref, rel)
        with open(p, "rb") as f:
            sha = hashlib.sha256(f.read()).hexdigest()
        fixture[rel] = {"sha256": sha, "values": reference_parse(p)}
    with open(os.path.join(HERE, "conf_shipped.json"), "w") as f:
        json.dump(fixture, f, indent=1, sort_keys=True)
    print("%d config files" % len(fixture))


if __name__ == "__main__":
    main()
