"""Generates tests/golden/checkpoint_gpu/ on a GPU: the reference's checkpoint
directory checkpoint_c1 with tiles 1 and 3 removed and then finished by
yar_gpu_render_checkpoint, plus checkpoint_gpu.npz with the image that call
returned.  The reference must resume from these files to the same image
(tests/test_checkpoint.py).  Run from the repository root on a GPU machine:

    python tests/golden/make_gpu_checkpoint.py [output directory]
"""
import os
import shutil
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from yar_gb300 import native  # noqa: E402
from yar_gb300.scene import FlatScene  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def main(out_root):
    out_dir = os.path.join(out_root, "checkpoint_gpu")
    shutil.rmtree(out_dir, ignore_errors=True)
    shutil.copytree(os.path.join(HERE, "checkpoint_c1"), out_dir)
    os.remove(os.path.join(out_dir, "tile_0001"))
    os.remove(os.path.join(out_dir, "tile_0003"))
    ctx = native.Context(0)
    ctx.upload_scene(FlatScene.read(os.path.join(HERE, "checkpoint_c1.yfs")))
    img, st = ctx.render_checkpoint(72, 72, out_dir, "cornell_checkpoint.pbrt")
    ctx.close()
    np.savez_compressed(os.path.join(out_root, "checkpoint_gpu.npz"), image=img, variance=np.float64(st.variance))
    print("wrote", out_dir)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
