"""Extract known-answer tests (KATs) from the reference's result logs.

Reads the CUNFFT result logs under ``<reference>/Tests/Runtime`` as text and
writes ``kats.json`` beside this script.  Each log line written by the
reference driver (Tests/Scripts/simpleTest.cpp:414-420) has the form

    [m, TX x TY] d l  t_nfft3 t_cundft t_cunfft | E_cundft E_nfft3

where ``l = log2(N_total)``, ``M = N_total`` (Tests/Scripts/test_cunfftRuntime.sh)
and ``E_cundft = ||cundft - cunfft||_inf / ||cundft||_inf`` (src/cuda_util.cpp:237-258),
i.e. the error of the reference's FP64 NFFT against its own direct NDFT.

Inputs behind each value: the reference driver fills the coefficients (f_hat
for the forward test, f for the adjoint test) with (drand48, drand48) pairs
and then the nodes with drand48() - 0.5 (src/cuda_util.cpp:151-171), from
glibc's unseeded stream (state 0).  The logged value belongs to the tenth of
ten repetitions in one process (the driver's 10-entry median arrays,
Tests/Scripts/simpleTest.cpp:55-56), so nine earlier draws of
``2*ncoef + M*d`` values precede the inputs.  ``skip_generations`` records that.

Only the E_cundft column is used: the NFFT3 column needs the third-party
NFFT3 library, which is absent.

Usage (in a checkout that has the reference tree):
    python tests/golden/make_kats.py /path/to/reference
"""
import json
import os
import re
import sys

LOGS = [
    ("Tests/Runtime/test_Runtime_m6.txt", "forward"),
    ("Tests/Runtime/test_Runtime_m12.txt", "forward"),
    ("Tests/Runtime/test_m6_ad.txt", "adjoint"),
    ("Tests/Runtime/test_m12_ad.txt", "adjoint"),
]
LINE = re.compile(
    r"^\s*\[(\d+),\s*(\d+)\s*x\s*(\d+)\]\s+(\d)\s+(\d+)\s+"
    r"([0-9.eE+-]+)\s+([0-9.eE+-]+)\s+([0-9.eE+-]+)\s*\|\s*([0-9.eE+-]+)\s+([0-9.eE+-]+)\s*$")


def parse(ref_root):
    kats, seen = [], {}
    for rel, direction in LOGS:
        with open(os.path.join(ref_root, rel)) as fh:
            for lineno, line in enumerate(fh, 1):
                mt = LINE.match(line)
                if not mt:
                    continue
                m, _tx, _ty, d, l = (int(mt.group(i)) for i in range(1, 6))
                t_cundft = float(mt.group(7))
                e_cundft = float(mt.group(9))
                if t_cundft == 0.0 or e_cundft == 0.0:
                    continue  # CUNDFT not run on this line
                if l % d:
                    continue
                n_dim = 1 << (l // d)
                key = (direction, m, d, l)
                if key in seen:
                    # the same configuration logged again with another thread-block size
                    prev = seen[key]
                    prev.setdefault("repeats", []).append({"file": rel, "line": lineno, "e_inf": e_cundft})
                    continue
                entry = {
                    "direction": direction, "m": m, "d": d, "N": [n_dim] * d,
                    "M": n_dim ** d, "e_inf": e_cundft, "skip_generations": 9,
                    "file": rel, "line": lineno,
                }
                seen[key] = entry
                kats.append(entry)
    return kats


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_kats.py <path of the CUNFFT source tree>")
    kats = parse(sys.argv[1])
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kats.json")
    with open(out, "w") as fh:
        json.dump({"source": "sukunis/CUNFFT Tests/Runtime logs (E_inf CUNDFT vs CUNFFT column)",
                   "generator": "tests/golden/make_kats.py", "kats": kats}, fh, indent=1)
    print(f"wrote {len(kats)} KATs to {out}")


if __name__ == "__main__":
    main()
