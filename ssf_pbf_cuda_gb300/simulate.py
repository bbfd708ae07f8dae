"""Headless main loop: the reference's src/main.cpp (a simulator step, then
the screen-space fluid frame, and the ms/frame printout once a second,
src/main.cpp:339-564) with the window replaced by device images, written as
binary PPM files when asked.

    python -m ssf_pbf_cuda_gb300.simulate --scene sphere --steps 600 --frame-every 20 --out frames
"""
from __future__ import annotations

import argparse
import os
import time


def main(argv=None) -> dict:
    from . import api
    from .simulators import SCENES

    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--scene", choices=sorted(SCENES), default="sphere")
    ap.add_argument("--space", type=float, default=None, help="particle spacing (default: the scene's own)")
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--frame-every", type=int, default=0, help="write a PPM frame every N steps (0: none)")
    ap.add_argument("--out", default="frames")
    ap.add_argument("--width", type=int, default=1280)
    ap.add_argument("--height", type=int, default=720)
    ap.add_argument("--no-render", action="store_true", help="simulate only")
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)

    kw = {"device": args.device}
    if args.space:
        kw["space"] = args.space
    sim = SCENES[args.scene](**kw)
    ren = None
    if not args.no_render:
        ren = api.SsfRenderer(api.ssf_default_params(width=args.width, height=args.height), device=args.device)
    if args.frame_every:
        os.makedirs(args.out, exist_ok=True)
    frames = []
    t_last, n_since = time.perf_counter(), 0
    for k in range(args.steps):
        sim.simulate_one_step()
        if ren is not None:
            ren.render_particles(sim.particle)
        n_since += 1
        if args.frame_every and (k + 1) % args.frame_every == 0 and ren is not None:
            path = os.path.join(args.out, f"{args.scene}_{k + 1:05d}.ppm")
            ren.save_ppm(path)
            frames.append(path)
        now = time.perf_counter()
        if now - t_last >= 1.0:
            num = sim.particles_num  # waits for the step, like the reference's printout
            now = time.perf_counter()
            print(f"{1000.0 * (now - t_last) / n_since:.3f} ms/frame")
            print(f"#particle: {num}")
            t_last, n_since = now, 0
    return {"steps": args.steps, "particles": sim.particles_num, "frames": frames}


if __name__ == "__main__":
    main()
