"""Regenerate the committed golden fixtures from the reference's own scripts.

Runs in the development container only (it needs the reference tree, which
does not travel with the repository):

    python tests/golden/make_golden.py [--ref /root/reference] [--max-floats N]

For each operator directory of the reference (fft1_d, rfft1_d, irfft1_d,
fft2_d) it imports ``tests/<op>_data/gen_data.py`` and
``tests/<op>_data/compare_data.py``, calls the reference's ``gen_one`` with
the reference's default seed (12345) inside a temporary directory, and copies
the resulting ``<case>_input.bin`` / ``<case>_golden.bin`` files (raw float32,
interleaved re/im for complex data) next to this script.  Cases whose files
exceed ``--max-floats`` are listed in the manifest as ``"skipped"`` and are
exercised at test time by regenerating inputs with the same recipe instead.
``manifest.json`` records each case's parameters, the reference tolerance
(atol, rtol) and the file names.
"""
from __future__ import annotations

import argparse
import contextlib
import importlib.util
import io
import json
import os
import shutil
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
OPS = ("fft1_d", "rfft1_d", "irfft1_d", "fft2_d")
SEED = 12345


def _load_module(path, name):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _case_floats(op, cfg):
    b = cfg.get("batch", 1)
    if op == "fft1_d":
        return 2 * cfg["n"] * b
    if op == "rfft1_d":
        return max(cfg["n"], 2 * (cfg["n"] // 2 + 1)) * b
    if op == "irfft1_d":
        return max(cfg["n"], 2 * (cfg["n"] // 2 + 1)) * b
    return 2 * cfg["fft_x"] * cfg["fft_y"] * b


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("OPS_FFT_REFERENCE", "/root/reference"))
    ap.add_argument("--max-floats", type=int, default=1 << 18)
    args = ap.parse_args()
    host = os.path.join(args.ref, "src", "common", "host")
    sys.path.insert(0, host)
    manifest = {"seed": SEED, "source": "reference src/<op>/tests/<op>_data/gen_data.py", "ops": {}}
    total_bytes = 0
    for op in OPS:
        data_dir = os.path.join(args.ref, "src", op, "tests", f"{op}_data")
        gen = _load_module(os.path.join(data_dir, "gen_data.py"), f"gen_{op}")
        cmp_ = _load_module(os.path.join(data_dir, "compare_data.py"), f"cmp_{op}")
        out_dir = os.path.join(HERE, op)
        os.makedirs(out_dir, exist_ok=True)
        cases = []
        for cfg in gen.configs:
            entry = dict(cfg)
            tol = cmp_.configs.get(cfg["name"])
            entry["atol"] = tol["atol"] if tol else None
            entry["rtol"] = tol["rtol"] if tol else None
            if _case_floats(op, cfg) > args.max_floats:
                entry["skipped"] = "too large to commit; regenerated at test time"
                cases.append(entry)
                continue
            with tempfile.TemporaryDirectory() as tmp:
                cwd = os.getcwd()
                os.chdir(tmp)
                try:
                    with contextlib.redirect_stdout(io.StringIO()):
                        gen.gen_one(cfg, SEED)
                finally:
                    os.chdir(cwd)
                files = {}
                for suffix in ("input", "golden", "golden_forward"):
                    src = os.path.join(tmp, f"{cfg['name']}_{suffix}.bin")
                    if os.path.exists(src):
                        dst = os.path.join(out_dir, os.path.basename(src))
                        shutil.copyfile(src, dst)
                        total_bytes += os.path.getsize(dst)
                        files[suffix] = os.path.basename(src)
            entry["files"] = files
            cases.append(entry)
        manifest["ops"][op] = cases
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    print(f"wrote {total_bytes / 1e6:.1f} MB of fixtures")


if __name__ == "__main__":
    main()
