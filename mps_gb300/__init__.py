"""GB300 (sm_103a) engine for the MPS (Moving Particle Semi-implicit) time step.

The compute path is the CUDA library behind include/mps_gb300.h; this
package holds its ctypes binding (engine.py), the build recipe (build.py),
the scene generator and CSV format (scenes.py) and the settings reader
(settings.py).  The C++ front end that mirrors the reference's
Simulation/MPS/Particle/Bucket classes lives in host/.
"""
from .engine import FP64, MIXED, Batch, Engine, MpsError, Trajectory, load, read_particles_csv, write_snapshot  # noqa: F401
