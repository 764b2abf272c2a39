"""Generates room_oracle.npz: the FP64-accumulated plain-mode render of the
hard-lighting room (yar_gb300.scenes.hard_lighting_room, 512 x 512, maxdepth
12) at PASSES one-sample passes, stored as float16 RGB.  It is the reference
image of the equal-time RMSE comparison of the guided render with the plain
one (bench.py --workload guided).  Runs on a GPU:

    python tests/golden/make_room_oracle.py [passes]
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from yar_gb300 import native, scenes  # noqa: E402

PASSES = int(sys.argv[1]) if len(sys.argv) > 1 else 65536
CHUNK = 1024


def main():
    s = scenes.hard_lighting_room()
    w, h = int(s.config["render_region"][2]), int(s.config["render_region"][3])
    ctx = native.Context(0)
    ctx.upload_scene(s)
    total = np.zeros((h, w, 3), np.float64)
    t = time.time()
    done = 0
    k = 0
    while done < PASSES:
        n = min(CHUNK, PASSES - done)
        _, sums, st = ctx.guided_render(w, h, passes=n, stream_offset=1000 + k)
        total += sums
        done += n
        k += 1
    img = total / done
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "room_oracle.npz")
    np.savez_compressed(out, image=img.astype(np.float16), passes=np.int64(done))
    print("room oracle: %d passes in %.1f s, mean %.6f -> %s" % (done, time.time() - t, img.mean(), out))


if __name__ == "__main__":
    main()
