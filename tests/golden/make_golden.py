"""Regenerate tests/golden/golden.json from the UNMODIFIED reference RendererSoft.

Runs every scene of tests/golden/cases.py through the reference-backed checker (oracle/_ref,
compiled from the reference sources by oracle/ref/Makefile; x86-64 with the reference tree only)
and records the SHA-256 prefixes of the scene inputs and of every attachment read back after the
frame. The fixture is committed; tests compare the CPU oracle (anywhere) and the CUDA renderer
(on a GPU) against it.

    python tests/golden/make_golden.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import oracle  # noqa: E402
from cases import CASES  # noqa: E402
from softglrender_gb300 import api as A  # noqa: E402
from softglrender_gb300 import scenes as S  # noqa: E402


def main():
    oracle.build()
    lib = oracle.reference()
    if lib is None:
        raise SystemExit("the reference checker is not available on this host")
    golden = {}
    for name in sorted(CASES):
        scene = CASES[name]()
        r = A.Renderer(lib, 0)
        inst = S.SceneInstance(r, scene)
        inst.render()
        outs = [S.output_digest(inst.outputs(i)) for i in range(len(scene.passes))]
        r.destroy()
        golden[name] = {"input": scene.input_digest(), "outputs": outs}
        print(name, golden[name])
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump({"generator": "reference RendererSoft (deterministic build, oracle/ref/Makefile)",
                   "cases": golden}, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
