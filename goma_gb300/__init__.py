"""GB300-native Q2/P1 Newton path (assembly, CSR scatter, Krylov solve)."""
from .problem import (Material, Mesh, Problem, box_mesh, boussinesq_cube_3d,  # noqa: F401
                      carreau_step_2d, lid_cavity_2d, make_desc, mesh_from_spec)
