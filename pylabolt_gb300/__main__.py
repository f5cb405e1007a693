"""``python -m pylabolt_gb300`` -- the reference's command line
(pylabolt/pylabolt.py:5-56) for the fluidLB solver on the GPU backend."""
from argparse import ArgumentParser


def main(argv=None):
    parser = ArgumentParser(description="A Lattice Boltzmann Python solver (GB300 fluidLB)")
    parser.add_argument("-s", "--solver", choices=["fluidLB", "phaseFieldLB", "cgLB"],
                        type=str, help="choice of solver to run")
    parser.add_argument("-b", "--backend", choices=["cpu", "gpu"], default="gpu",
                        type=str, help="choice of backend: CPU/GPU (CUDA)")
    parser.add_argument("-nt", "--n_threads", type=int, default=1,
                        help="Number of threads for OpenMP/CUDA")
    parser.add_argument("--reconstruct", choices=["all", "time", None], default=None,
                        help="Domain reconstruction")
    parser.add_argument("-t", "--time", type=int, default=0,
                        help="Specify time which is to be reconstructed")
    parser.add_argument("--to_vtk", choices=["all", "time", None], default=None,
                        help="Convert output data to VTK format")
    parser.add_argument("--debug", action="store_true", default=False,
                        help="Run in debug mode")
    args = parser.parse_args(argv)
    if args.solver == "fluidLB":
        from .solver import main as run
        run(args.backend, args.n_threads, debug_mode=args.debug)
    elif args.solver is not None:
        raise SystemExit(f"solver {args.solver} is not provided by pylabolt_gb300")
    if args.reconstruct is not None or args.to_vtk is not None:
        # one rank writes global fields: nothing to reconstruct; VTK
        # conversion reads output/fields with the reference's own tool
        raise SystemExit("--reconstruct / --to_vtk: run the reference's post-processing "
                         "on output/ (this package writes its layout)")


if __name__ == "__main__":
    main()
