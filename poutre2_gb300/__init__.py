"""poutre2_gb300 -- GB300-native (sm_103a) morphology + geodesy hot path of poutre2.

The compute path is one C-ABI shared library (``_build/libpoutre_gb300.so``, built
from ``csrc/``) of hand-written CUDA kernels.  The Python modules mirror poutre2's
public API on device images (torch CUDA tensors) and call that library through
ctypes; there is no CPU fallback: every entry point raises if the library or a GPU
is missing.

Modules: ``llm`` (erosion / dilation, openings, lines), ``geo`` (reconstruction, h-extrema,
leveling, the ragged h-maxima batch), ``label`` (connected components, labelled extrema),
``pixel`` (arithmetic, CompareImage, conversion), ``autograd`` (flat-morphology adjoint),
``pypoutre`` (the nanobind module's own names), ``image`` / ``se`` (images, SEs).
"""
from .se import Common_NL_SE, Compound_NL_SE, NeighborList, predefined_offsets  # noqa: F401
