"""fdfk2d_gb300: GB300 (sm_103a) hot path of FDFK2D's hybrid FD-FK solver.

The compute runs in ``_build/libfdfk_gb300.so`` (hand-written CUDA, C ABI in
``include/fdfk_gb300.h``); this package is its host-side mirror of the
reference interface:

* :func:`updatedispl` - the reference's per-step entry point
  (``updatedispl_``, src/FDFK2D.f90:516-522), same arrays, same in-place update;
* :class:`Session` - device-resident solver state for the time loop of
  ``simulate_wavefield`` (src/FDFK2D.f90:465-532);
* :func:`simulate` - the whole time loop in one call (host arrays in, seismograms out);
* :class:`Batch` - many sessions advanced together (three launches per step for
  all of them, CUDA-graph replay);
* :func:`run` - program FDFK2D itself: the reference's input folder in (:func:`read_input`),
  SU seismograms out (:func:`write_su`), everything between on the GPU;
* :class:`Server` - the serving loop: requests admitted by device-memory budget
  into a running batch (continuous batching), retired when done;
* :func:`fk_background` / :func:`comput_background_wavefield` - the FK background
  (libFK3D's ``comput_background_wavefield_``, src/FDFK2D.f90:429-431) on the GPU,
  and :meth:`Session.fk_background` straight into a session's device strips.

There is no CPU fallback: if the CUDA library is missing or no GPU is
visible, calls raise.
"""
from .api import (Batch, FDFKError, FkParams, Params, Server, Session, autotune, backazimuths, read_input, read_su, run,
                  receiver_functions,
                  session_device_bytes, stable_dt, write_su, STRIPS, BP, BU, comput_background_wavefield,
                  fk_background, lib, lib_path, simulate, strip_shapes, pml_shapes, updatedispl, kernel_launches)

__all__ = ["Batch", "FDFKError", "Server", "autotune", "backazimuths", "read_input", "read_su", "receiver_functions", "run",
           "session_device_bytes",
           "stable_dt", "write_su", "FkParams", "Params", "Session", "STRIPS", "BP", "BU", "comput_background_wavefield",
           "fk_background", "lib", "lib_path", "simulate", "strip_shapes", "pml_shapes", "updatedispl",
           "kernel_launches"]
