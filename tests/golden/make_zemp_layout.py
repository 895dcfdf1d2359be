"""Generate tests/golden/zemp_bp_v1_layout.json: size and field offsets of the
reference's dataset parameter block (zemp_bp_v1, tests/throughput.c), printed by
oracle/_ref/zemp_probe, a probe compiled by oracle/build_ref.py from the typedef
in the reference's own source.

Usage: python oracle/build_ref.py && python tests/golden/make_zemp_layout.py
"""
import json
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
def main():
    probe = os.path.normpath(os.path.join(HERE, "..", "..", "oracle", "_ref", "zemp_probe"))
    if not os.path.exists(probe):
        raise SystemExit("oracle/_ref/zemp_probe is not built (python oracle/build_ref.py)")
    out = subprocess.run([probe], check=True, capture_output=True, text=True).stdout
    layout = {}
    for line in out.splitlines():
        name, value = line.split()
        layout[name] = int(value)
    with open(os.path.join(HERE, "zemp_bp_v1_layout.json"), "w") as f:
        json.dump(layout, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
