"""Writes tests/golden/imf_powerlaw_bins.txt: the reference's own known-answer table of power-law IMF bin
integrals, produced by running the reference's generator (tools/reference/imf_powerlaw_bins.py in the OpenSPS tree:
60-digit Python decimal integrals of m^-alpha over bins chosen where a difference of powers breaks).

Usage: python tests/golden/make_imf_kat.py /path/to/opensps-source   (or OPENSPS_SOURCE_DIR set)
"""
import os
import subprocess
import sys
from pathlib import Path

if len(sys.argv) > 1:
    src = Path(sys.argv[1])
elif os.environ.get("OPENSPS_SOURCE_DIR"):
    src = Path(os.environ["OPENSPS_SOURCE_DIR"])
else:
    sys.exit("usage: make_imf_kat.py /path/to/opensps-source (or set OPENSPS_SOURCE_DIR)")
out = Path(__file__).resolve().parent / "imf_powerlaw_bins.txt"
text = subprocess.run([sys.executable, str(src / "tools" / "reference" / "imf_powerlaw_bins.py")],
                      check=True, capture_output=True, text=True).stdout
out.write_text(text)
print(out, len(text.splitlines()), "lines")
