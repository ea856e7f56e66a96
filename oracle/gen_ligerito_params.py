"""Generates the Ligerito parameter tables from the reference's embedded TOMLs.

Usage: python oracle/gen_ligerito_params.py REFERENCE_ROOT

Reads crates/flock-core/configs/ligerito/m{22..35}_{fast,slim,secure}.toml of
the reference tree (REFERENCE_ROOT, required) and writes the same numbers as C
initializers into flock_challenge_gb300/csrc/ligerito_params.inc, which both
the product library and the oracle include.
Row: m, profile (0 fast, 1 slim, 2 secure), initial_k, yr_log_n, n_levels,
then per level {log_inv_rate, log_msg_cols, log_num_interleaved, k_recursive,
queries, grinding_bits, fold_grinding_bits, ood_samples}.
These are protocol constants (query counts, grinding bits, rates) that must
match the reference exactly, so they are copied, not re-derived.
"""
import os
import re
import sys

if len(sys.argv) != 2:
    raise SystemExit(__doc__)
ref = sys.argv[1]
here = os.path.dirname(os.path.abspath(__file__))
cfg_dir = os.path.join(ref, "crates/flock-core/configs/ligerito")
KEYS = ["log_inv_rate", "log_msg_cols", "log_num_interleaved", "k_recursive", "queries", "grinding_bits",
        "fold_grinding_bits", "ood_samples"]
rows = []
for m in range(22, 36):
    for pi, prof in enumerate(["fast", "slim", "secure"]):
        path = os.path.join(cfg_dir, f"m{m}_{prof}.toml")
        if not os.path.exists(path):
            continue
        txt = open(path).read()
        head, *levels = re.split(r"\[\[levels\]\]", txt)
        levels[-1], final = levels[-1].split("[final_block]")

        def num(block, key):
            mm = re.search(rf"^{key}\s*=\s*(\d+)", block, re.M)
            assert mm, (path, key)
            return int(mm.group(1))
        init_k = num(head, "initial_k")
        yr = num(final, "yr_log_n")
        lv = [[num(b, k) for k in KEYS] for b in levels]
        rows.append((m, pi, init_k, yr, lv))

max_levels = max(len(r[4]) for r in rows)
out = ["// Generated by oracle/gen_ligerito_params.py from the reference's",
       "// crates/flock-core/configs/ligerito/*.toml. Do not edit by hand.",
       f"#define LIGERITO_MAX_LEVELS {max_levels}",
       f"#define LIGERITO_N_CONFIGS {len(rows)}",
       "static const int LIGERITO_CONFIGS[LIGERITO_N_CONFIGS][4 + 1 + LIGERITO_MAX_LEVELS * 8] = {"]
for m, pi, k, yr, lv in rows:
    flat = [m, pi, k, yr, len(lv)]
    for L in lv:
        flat += L
    flat += [0] * (8 * (max_levels - len(lv)))
    out.append("  {" + ", ".join(map(str, flat)) + "},")
out.append("};")
text = "\n".join(out) + "\n"
for dst in [os.path.join(os.path.dirname(here), "flock_challenge_gb300", "csrc", "ligerito_params.inc")]:
    open(dst, "w").write(text)
    print("wrote", dst, len(rows), "configs")
