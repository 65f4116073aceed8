"""Writes tests/golden/imf_powerlaw_bins.txt: the reference's own known-answer table of power-law IMF bin
integrals, produced by running the reference's generator (tools/reference/imf_powerlaw_bins.py in the OpenSPS tree:
60-digit Python decimal integrals of m^-alpha over bins chosen where a difference of powers breaks).

Usage: python tests/golden/make_imf_kat.py /path/to/opensps-source
"""
import subprocess
import sys
from pathlib import Path

src = Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
out = Path(__file__).resolve().parent / "imf_powerlaw_bins.txt"
text = subprocess.run([sys.executable, str(src / "tools" / "reference" / "imf_powerlaw_bins.py")],
                      check=True, capture_output=True, text=True).stdout
out.write_text(text)
print(out, len(text.splitlines()), "lines")
