"""CPU: the compiled stride table (femtc_gb300/csrc/slab_strides.hpp) is what
its generator (slab_strides_gen.cpp, the bank-conflict cost model) prints."""
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "femtc_gb300", "csrc")


def test_stride_table_matches_generator(tmp_path):
    exe = str(tmp_path / "gen")
    subprocess.run(["g++", "-O2", os.path.join(CSRC, "slab_strides_gen.cpp"), "-o", exe],
                   check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    gen = re.findall(r"\{([-\d, ]+)\}", out)
    txt = open(os.path.join(CSRC, "slab_strides.hpp")).read()
    table = txt[txt.index("kSlabStrides[] = {"):]
    table = table[:table.index("};")]
    have = re.findall(r"\{([-\d, ]+)\}", table)
    norm = lambda rows: [tuple(int(x) for x in r.split(",")) for r in rows]
    assert norm(gen) == norm(have)
    # every slab variant of the library (N 2..8, Q N..N+2, 4- and 8-byte
    # values, 1 or 2 lanes) has an entry
    keys = {r[:4] for r in norm(have)}
    for n in range(2, 9):
        for q in range(n, n + 3):
            for es in (4, 8):
                for lanes in (1, 2):
                    assert (n, q, es, lanes) in keys
