"""Command line renderer: ``python -m radiantiumplusplus_gb300 --scene scene.json``.

The flow of the reference's CLI (rad.offline.cli/main.cpp:8-80) on the GPU
library: ``--scene`` names the JSON scene (resolved as given, else against the
working directory), the scene is built, a progress line (elapsed time, total and
completed pixel tasks) is printed every second while the job runs, and the film
is saved as ``<scene directory>/<scene file stem>.exr``. Extra switches, which
the reference lacks: ``--spp`` overrides the sampler's sample count, ``--out``
the output path, ``--guide`` samples with the scene's learned proposal.
"""

from __future__ import annotations

import os
import sys
import threading
import time


def _parse(argv):
    opts = {"scene": None, "spp": 0, "out": None, "guide": False}
    i = 0
    while i < len(argv):
        a = argv[i]
        if a in ("--scene", "--spp", "--out") and i + 1 < len(argv):
            opts[a[2:]] = argv[i + 1] if a != "--spp" else int(argv[i + 1])
            i += 2
        elif a == "--guide":
            opts["guide"] = True
            i += 1
        else:
            i += 1
    return opts


def main(argv=None):
    opts = _parse(sys.argv[1:] if argv is None else argv)
    if not opts["scene"]:
        print('error: should input cmd like "--scene <scene.json>"', file=sys.stderr)
        return 2
    path = opts["scene"]
    if not os.path.exists(path):
        work = os.path.join(os.getcwd(), path)
        if not os.path.exists(work):
            print("error: cannot open file: %s" % path, file=sys.stderr)
            return 2
        path = work
    import radiantiumplusplus_gb300 as rad
    from .exr import write_exr
    try:
        scene = rad.Scene.from_file(path)
        print("start rendering...", flush=True)
        t0 = time.perf_counter()
        job = scene.submit(spp=opts["spp"], guide=opts["guide"])
        done = threading.Event()

        def bar():
            while not done.wait(1.0):
                d, total = job.progress()
                npix = scene.width * scene.height
                spp = max(1, total // max(1, npix))
                print("\r[%8.1f s] %d / %d pixels" % (time.perf_counter() - t0, d // spp, npix), end="", flush=True)

        th = threading.Thread(target=bar, daemon=True)
        th.start()
        try:
            job.wait()
        finally:
            done.set()
            th.join()
            print("", flush=True)
        film = job.film()
        out = opts["out"] or os.path.join(os.path.dirname(os.path.abspath(path)),
                                          os.path.splitext(os.path.basename(path))[0] + ".exr")
        write_exr(out, film)
        print("save result to: %s" % out)
        print("done. render used time: %d ms" % int((time.perf_counter() - t0) * 1000), flush=True)
        job.close()
        scene.close()
    except rad.RadError as e:
        print("error: %s" % e, file=sys.stderr)
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
