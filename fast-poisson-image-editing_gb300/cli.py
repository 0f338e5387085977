"""Command line, mirroring the reference's ``fpie`` (fpie/cli.py, fpie/args.py).

    python -m fpie_gb300.cli -s src.png -m mask.png -t tgt.png -o out.png \\
        -h0 0 -w0 0 -h1 100 -w1 100 -n 5000 -g max --method grid -b gb300

Same flags and prints as the reference; ``--check-backend`` lists
``ALL_BACKEND`` (the gb300 backends) and exits.  ``-p P`` writes
``iterNNNNN.png`` every P sweeps, as the reference does.  The solver inputs
are built on the GPU from the uint8 images (bit-identical to the host
construction, which takes 0.1-0.2 s with numpy on a 1024^2 target);
``--host-prep`` builds them on the host as the reference does.
"""

from __future__ import annotations

import argparse
import os
import sys
import time

from . import __version__
from .process import ALL_BACKEND, BACKEND_NOTES, CPU_COUNT, DEFAULT_BACKEND


def get_args(argv=None) -> argparse.Namespace:
    """Arguments of the command line (fpie/args.py:10-142, 'cli' flavour)."""
    p = argparse.ArgumentParser(prog="fpie_gb300")
    p.add_argument("-v", "--version", action="store_true", help="show the version and exit")
    p.add_argument("--check-backend", action="store_true", help="print all available backends")
    p.add_argument("-b", "--backend", type=str, choices=ALL_BACKEND, default=DEFAULT_BACKEND,
                   help="backend choice")
    p.add_argument("-c", "--cpu", type=int, default=CPU_COUNT, help="number of CPU used")
    p.add_argument("-z", "--block-size", type=int, default=1024,
                   help="cuda block size (only for equ solver)")
    p.add_argument("--method", type=str, choices=["equ", "grid"], default="equ",
                   help="how to parallelize computation")
    p.add_argument("-s", "--source", type=str, help="source image filename")
    p.add_argument("-m", "--mask", type=str, default="",
                   help="mask image filename (default is to use the whole source image)")
    p.add_argument("-t", "--target", type=str, help="target image filename")
    p.add_argument("-o", "--output", type=str, help="output image filename")
    p.add_argument("-h0", type=int, default=0, help="mask position (height) on source image")
    p.add_argument("-w0", type=int, default=0, help="mask position (width) on source image")
    p.add_argument("-h1", type=int, default=0, help="mask position (height) on target image")
    p.add_argument("-w1", type=int, default=0, help="mask position (width) on target image")
    p.add_argument("-g", "--gradient", type=str, choices=["max", "src", "avg"], default="max",
                   help="how to calculate gradient for PIE")
    p.add_argument("-n", type=int, default=5000,
                   help="how many iteration would you perfer, the more the better")
    p.add_argument("-p", type=int, default=0, help="output result every P iteration")
    p.add_argument("--grid-x", type=int, default=8, help="x axis stride for grid solver")
    p.add_argument("--grid-y", type=int, default=8, help="y axis stride for grid solver")
    p.add_argument("--device-prep", dest="device_prep", action="store_true", default=True,
                   help="build the solver inputs on the GPU from the uint8 images (default)")
    p.add_argument("--host-prep", dest="device_prep", action="store_false",
                   help="build the solver inputs on the host with numpy, as the reference does")
    args = p.parse_args(argv)
    if args.version:
        print(__version__)
        sys.exit(0)
    if args.check_backend:
        print(ALL_BACKEND)
        for name in ALL_BACKEND:
            print(f"  {name}: {BACKEND_NOTES[name]}")
        sys.exit(0)
    for name, path in (("Source", args.source), ("Target", args.target)):
        if not path or not os.path.exists(path):
            print(f"{name} image {path} not found.")
            sys.exit(1)
    return args


def main(argv=None) -> None:
    args = get_args(argv)
    from .io import read_images, write_image
    from .process import EquProcessor, GridProcessor

    if args.method == "equ":
        proc = EquProcessor(args.gradient, args.backend, args.cpu, 100, args.block_size,
                            device_prep=args.device_prep)
    else:
        proc = GridProcessor(args.gradient, args.backend, args.cpu, 100, args.block_size,
                             args.grid_x, args.grid_y, device_prep=args.device_prep)
    print(f"Successfully initialize PIE {args.method} solver with {args.backend} backend")
    src, mask, tgt = read_images(args.source, args.mask, args.target)
    n = proc.reset(src, mask, tgt, (args.h0, args.w0), (args.h1, args.w1))
    print(f"# of vars: {n}")
    proc.sync()
    result = tgt
    t = time.time()
    p = args.p or args.n
    for i in range(0, args.n, p):
        result, err = proc.step(p)
        print(f"Iter {i + p}, abs error {err}")
        if i + p < args.n:
            write_image(f"iter{i + p:05d}.png", result)
    print(f"Time elapsed: {time.time() - t:.4f}s")
    write_image(args.output, result)
    print(f"Successfully write image to {args.output}")


if __name__ == "__main__":
    main()
