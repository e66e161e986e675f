"""Exodus II results files of converged solutions (host side).

The reference writes its solutions with wr_exo.c / wr_soln.c through the
Exodus II library.  This writer produces the same content for the meshes
and fields of this package, so a GPU solution opens in the tools that
read the reference's output:

- nodal variables VX, VY, (VZ), (T), (Y0, Y1, ...) -- the names of
  include/mm_names.h:7670-7679, species as "Y<k>" when unnamed
  (src/rf_vars.c:594);
- the discontinuous P1 pressure as element variables P_E0 .. P_E<dim>, one
  per pressure coefficient of the element, as the reference does for I_P1
  fields (src/mm_post_proc.c:12347-12355, src/wr_exo.c:924-930);
- one element block (QUAD9 or HEX27, connectivity in the element's local
  node order, 1-based), node sets, and one record per time step (a
  continuation parameter may stand in for time).

The file is NetCDF classic with 64-bit offsets in the Exodus II layout:
"large model" coordinates coordx/coordy/coordz, connect1 with an elem_type
attribute, vals_nod_var<i>(time_step, num_nodes) and
vals_elem_var<j>eb1(time_step, num_el_in_blk1) with a truth table, names
in character arrays of len_name = 33.  The NetCDF encoding is SciPy's
netcdf_file.

The unknowns of a solution vector follow the library's DOF map: per node,
in node order, the nodal fields (u, v, (w), (T), (Y_0 ...)), and at the
centroid node of each element (local node 8 of QUAD9, 20 of HEX27) the
element's dim + 1 pressure coefficients after them.
"""
import numpy as np

LEN_NAME = 33
LEN_LINE = 81


def first_unknowns(problem):
    """First unknown of every node (num_nodes + 1), the library's DOF map."""
    mesh = problem.mesh
    dim = problem.dim
    nvn = dim + (1 if problem.energy else 0) + problem.num_species
    counts = np.full(mesh.num_nodes, nvn, np.int64)
    centroid = mesh.conn[:, 8 if dim == 2 else 20]
    counts[centroid] += dim + 1
    fu = np.zeros(mesh.num_nodes + 1, np.int64)
    np.cumsum(counts, out=fu[1:])
    return fu


def field_names(problem):
    """Nodal and element variable names of the reference's output."""
    dim = problem.dim
    nodal = ["VX", "VY", "VZ"][:dim]
    if problem.energy:
        nodal.append("T")
    nodal += ["Y%d" % k for k in range(problem.num_species)]
    elem = ["P_E%d" % k for k in range(dim + 1)]
    return nodal, elem


def split_solution(problem, x):
    """(nodal values (num_nodal_fields, num_nodes), element pressure
    coefficients (dim + 1, num_elems)) of a solution vector."""
    mesh = problem.mesh
    x = np.asarray(x, np.float64)
    fu = first_unknowns(problem)
    if x.shape != (fu[-1],):
        raise ValueError("solution has %d unknowns, the mesh %d" % (x.shape[0], fu[-1]))
    nodal_names, elem_names = field_names(problem)
    nodal = np.stack([x[fu[:-1] + k] for k in range(len(nodal_names))])
    nvn = len(nodal_names)
    centroid = mesh.conn[:, 8 if problem.dim == 2 else 20]
    elem = np.stack([x[fu[centroid] + nvn + k] for k in range(len(elem_names))])
    return nodal, elem


def _chars(strings, width):
    out = np.zeros((len(strings), width), "S1")
    for i, s in enumerate(strings):
        b = s.encode()[:width - 1]
        out[i, :len(b)] = np.frombuffer(b, "S1")
    return out


class ExodusWriter:
    """Exodus II results file: the mesh once, then write_step() per solution."""

    def __init__(self, path, problem, title="goma_gb300 solution"):
        from scipy.io import netcdf_file
        mesh = problem.mesh
        self.problem = problem
        dim = problem.dim
        ne, nn = mesh.num_elems, mesh.num_nodes
        npe = mesh.conn.shape[1]
        nodal_names, elem_names = field_names(problem)
        f = netcdf_file(path, "w", version=2)
        self.f = f
        f.api_version = np.float32(8.03)
        f.version = np.float32(8.03)
        f.floating_point_word_size = np.int32(8)
        f.file_size = np.int32(1)
        f.maximum_name_length = np.int32(LEN_NAME - 1)
        f.int64_status = np.int32(0)
        f.title = title[:LEN_LINE - 1]
        f.createDimension("time_step", None)  # the record dimension comes first
        for name, size in (("len_string", LEN_NAME), ("len_name", LEN_NAME),
                           ("len_line", LEN_LINE), ("four", 4), ("num_dim", dim),
                           ("num_nodes", nn), ("num_elem", ne), ("num_el_blk", 1),
                           ("num_el_in_blk1", ne), ("num_nod_per_el1", npe),
                           ("num_nod_var", len(nodal_names)),
                           ("num_elem_var", len(elem_names))):
            f.createDimension(name, size)
        f.createVariable("time_whole", "d", ("time_step",))
        for a, c in zip("xyz", range(dim)):
            v = f.createVariable("coord" + a, "d", ("num_nodes",))
            v[:] = mesh.coords[:, c]
        f.createVariable("coor_names", "c", ("num_dim", "len_name"))[:] = _chars(
            ["x", "y", "z"][:dim], LEN_NAME)
        f.createVariable("eb_status", "i", ("num_el_blk",))[:] = np.array([1], np.int32)
        prop = f.createVariable("eb_prop1", "i", ("num_el_blk",))
        prop[:] = np.array([1], np.int32)
        prop.name = "ID"
        f.createVariable("eb_names", "c", ("num_el_blk", "len_name"))[:] = _chars(
            ["block_1"], LEN_NAME)
        conn = f.createVariable("connect1", "i", ("num_el_in_blk1", "num_nod_per_el1"))
        conn[:] = (mesh.conn + 1).astype(np.int32)
        conn.elem_type = "QUAD9" if dim == 2 else "HEX27"
        sets = [np.asarray(s, np.int64) for s in mesh.node_sets]
        if sets:
            f.createDimension("num_node_sets", len(sets))
            f.createVariable("ns_status", "i", ("num_node_sets",))[:] = np.ones(
                len(sets), np.int32)
            nsp = f.createVariable("ns_prop1", "i", ("num_node_sets",))
            nsp[:] = np.arange(1, len(sets) + 1, dtype=np.int32)
            nsp.name = "ID"
            for k, s in enumerate(sets):
                f.createDimension("num_nod_ns%d" % (k + 1), len(s))
                f.createVariable("node_ns%d" % (k + 1), "i", ("num_nod_ns%d" % (k + 1),))[:] = (
                    s + 1).astype(np.int32)
        f.createVariable("name_nod_var", "c", ("num_nod_var", "len_name"))[:] = _chars(
            nodal_names, LEN_NAME)
        f.createVariable("name_elem_var", "c", ("num_elem_var", "len_name"))[:] = _chars(
            elem_names, LEN_NAME)
        f.createVariable("elem_var_tab", "i", ("num_el_blk", "num_elem_var"))[:] = np.ones(
            (1, len(elem_names)), np.int32)
        self.nodal = [f.createVariable("vals_nod_var%d" % (i + 1), "d", ("time_step", "num_nodes"))
                      for i in range(len(nodal_names))]
        self.elem = [f.createVariable("vals_elem_var%deb1" % (j + 1), "d",
                                      ("time_step", "num_el_in_blk1"))
                     for j in range(len(elem_names))]
        self.steps = 0

    def write_step(self, time, x):
        """One record: the solution x (the library's unknown order) at time."""
        nodal, elem = split_solution(self.problem, x)
        k = self.steps
        self.f.variables["time_whole"][k] = time
        for v, vals in zip(self.nodal, nodal):
            v[k] = vals
        for v, vals in zip(self.elem, elem):
            v[k] = vals
        self.steps += 1

    def close(self):
        self.f.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def write_exodus(path, problem, solutions, times=None, title="goma_gb300 solution"):
    """Writes one or more solution vectors (e.g. the steps of a
    continuation, times = the parameter values) to an Exodus II file."""
    if isinstance(solutions, np.ndarray) and solutions.ndim == 1:
        solutions = [solutions]
    times = list(times) if times is not None else list(range(len(solutions)))
    with ExodusWriter(path, problem, title) as w:
        for t, x in zip(times, solutions):
            w.write_step(float(t), x)
