"""The small seeded problems of the golden fixtures (oracle outputs committed
under tests/golden/): name -> (problem builder, steps, well-balanced).  The
builders are the ones the parity tests use, at sizes the oracle runs in well
under a second."""
import os
import sys

sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))
from problems import polytrope_2d, polytrope_3d, vortex_2d, vortex_tube_3d  # noqa: E402

CASES = {
    "vortex2d_hllc_n12": (lambda: vortex_2d(n=12, halo=3, flux=0), 5, False),
    "vortex2d_rusanov_n12": (lambda: vortex_2d(n=12, halo=3, flux=1), 5, False),
    "polytrope2d_r12": (lambda: polytrope_2d(n_rings=12, amplitude=1e-2, seed=3), 3, True),
    "tube3d_o3_n5": (lambda: vortex_tube_3d(n=5), 3, False),
    "tube3d_o2_n5": (lambda: vortex_tube_3d(n=5, order=2), 3, False),
    "polytrope3d_n5": (lambda: polytrope_3d(n=5, amplitude=1e-2), 3, True),
}
