"""2-D square-lattice networks (PEPS / PEPO) on the GPU."""
from .square_lattice import *  # noqa: F401,F403
