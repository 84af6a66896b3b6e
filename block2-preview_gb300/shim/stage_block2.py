"""Stages block2's headers for building the drop-in where block2 is not installed.

block2 is a header-only C++ library: the sweep program (dmrg_sweep.cpp) and
the drop-in (b2g_block2.hpp) compile against its src/ tree.  A machine that
has no block2 checkout (the Arm GPU host runs from a copy of this working
tree) gets one from this script: it copies block2_core.hpp, block2_dmrg.hpp
and the core/ and dmrg/ headers they include, unchanged, into
shim/_block2/src (git-ignored; nothing of block2 is committed here).

    python stage_block2.py BLOCK2_SRC_DIR
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
STAGED = os.path.join(HERE, "_block2", "src")


def stage(src: str) -> str:
    if not os.path.isfile(os.path.join(src, "block2_core.hpp")):
        raise FileNotFoundError(f"no block2 source tree at {src}")
    tmp = STAGED + ".tmp"
    if os.path.isdir(tmp):
        shutil.rmtree(tmp)
    os.makedirs(tmp)
    for f in ("block2_core.hpp", "block2_dmrg.hpp"):
        shutil.copy2(os.path.join(src, f), os.path.join(tmp, f))
    for d in ("core", "dmrg"):
        os.makedirs(os.path.join(tmp, d))
        for f in sorted(os.listdir(os.path.join(src, d))):
            if f.endswith(".hpp"):
                shutil.copy2(os.path.join(src, d, f), os.path.join(tmp, d, f))
    if os.path.isdir(STAGED):
        shutil.rmtree(STAGED)
    os.replace(tmp, STAGED)
    return STAGED


if __name__ == "__main__":
    print(stage(sys.argv[1]))
