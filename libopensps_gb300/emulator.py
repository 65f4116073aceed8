"""The learned emulator's weights: training them on this library's CSP and finding the file the library ships.

    python -m libopensps_gb300.emulator train [--out PATH] [--n-train N] [--n-val N] [--epochs E] [--batch B]
                                              [--seed S]

trains the ensemble (opensps_gb300_emulator_train) on the synthetic data root with the operator dataset, the 40
Gaussian filters, IGM absorption and the delayed-tau SFH, and writes the weights file. The defaults are the
shipped file's settings: 4,194,304 training models (seed 1) and 32,768 validation models.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time
from pathlib import Path

WEIGHTS = Path(__file__).resolve().parent / "emulator_data" / "gauss40_ops_sfh4.emu"


def training_context():
    """A context set up as the shipped emulator's training: synthetic libraries, 40 Gaussian filters, IGM on, the
    SSP operators built, sfh = 4."""
    from . import synthdata
    from .capi import Context
    root = synthdata.default_root()
    synthdata.generate(root)
    os.environ["OPENSPS_DATA_HOME"] = str(root)
    c = Context()
    c.set_int("add_igm_absorption", 1)
    c.build_ssp_ops()
    c.set_int("sfh", 4)
    return c


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m libopensps_gb300.emulator")
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--out", default=str(WEIGHTS))
    t.add_argument("--n-train", type=int, default=4194304)
    t.add_argument("--n-val", type=int, default=32768)
    t.add_argument("--epochs", type=int, default=60)
    t.add_argument("--batch", type=int, default=8192)
    t.add_argument("--seed", type=int, default=1)
    a = ap.parse_args(argv)
    out = Path(a.out)
    out.parent.mkdir(parents=True, exist_ok=True)
    c = training_context()
    t0 = time.time()
    c.emulator_train(out, n_train=a.n_train, n_val=a.n_val, epochs=a.epochs, batch=a.batch, seed=a.seed)
    info = c.emulator_info()
    info["wall_s"] = time.time() - t0
    print(json.dumps(info))
    c.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
