"""citrus_gb300: the CITRUS scatter step on GB300 (sm_103a).

The host side mirrors ``citrus.scatter_solver``'s call surface (grids, geometry, direction sets, the sweep context,
source iteration, ray tracing, the uncollided fluence and first-collision source, the collapsed-cone scatter image
and the per-view CITRUS step); every numerical kernel is a hand-written CUDA kernel in ``libcitrus_gb300.so``, called
through its C ABI (``include/citrus_gb300.h``). There is no CPU or Triton path.

Beyond the reference: ``batched`` runs the views of an outer iteration with their sweeps batched and replays the whole
iteration from a CUDA graph, ``autotune`` picks launch shapes by timing them on the device, ``learned`` trains and runs
the 3D U-Net that proposes the higher collision orders of a cold-start accumulator, and ``state_store`` and
``density`` carry the CITRUS loop's per-view state and density model.
"""

__version__ = "0.1.0"
