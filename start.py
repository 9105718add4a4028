"""Command line: ``python start.py <app_name> [precision]`` (as lbm's start.py)."""
import sys

from lbm_gb300 import app_factory, lattice, run

if __name__ == "__main__":
    if len(sys.argv) not in (2, 3):
        print("Command line error, please use as follows:")
        print("python3 start.py app_name [q60|f64|f32|f16s|f16sr|bf16s|bf16sr]")
        sys.exit(1)
    app = app_factory.create(sys.argv[1])
    ltc = lattice(app, precision=sys.argv[2] if len(sys.argv) == 3 else None)
    run(ltc, app)
