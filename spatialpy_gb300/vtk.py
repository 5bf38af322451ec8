"""VTK legacy ASCII writer for engine outputs.

Writes ``outputN.vtk`` files in the layout the reference engine produces
(spatialpy/solvers/c_base/ssa_sdpd-c-simulation-engine/src/output.cpp:104-229),
so ``spatialpy.core.vtkreader.VTKReader`` and other VTK tools read GPU results:
POLYDATA points at ``%.10e`` (3 per line), one VERTEX per point, then a FIELD
block with ``id``, ``type``, ``v``, ``rho``, ``mass``, ``bvf_phi``, ``nu``
(``%lf``, i.e. 6 decimals; 9 values per line, vectors 3 per line) and one
``D[species]`` int array per stochastic species.  The FIELD count of output 0
omits the species arrays, as the reference's does (its RDME state is not yet
initialised when output 0 is written, output.cpp:151-158), though the arrays
follow.
"""
from __future__ import annotations

import os

import numpy as np


def _rows(values, per_line, fmt):
    out = []
    for i, v in enumerate(values):
        out.append(fmt % v)
        if (i + 1) % per_line == 0:
            out.append("\n")
    return "".join(out)


def _vec_rows(arr, fmt):
    out = []
    for i, row in enumerate(arr):
        out.append((fmt + " " + fmt + " " + fmt + " ") % (row[0], row[1], row[2]))
        if (i + 1) % 3 == 0:
            out.append("\n")
    return "".join(out)


def format_step(points, types, v, rho, mass, bvf_phi, nu, species, counts, index, chem=None):
    """One output file as text.  counts: [N, S] copy numbers; chem: [N, S]
    deterministic concentrations or None (output.cpp writes them as C[s])."""
    n = points.shape[0]
    parts = ["# vtk DataFile Version 4.1\n", "Generated by SpatialPy\n", "ASCII\n",
             "DATASET POLYDATA\n", f"POINTS {n} float\n",
             _vec_rows(points, "%.10e"), "\n",
             f"VERTICES {n} {2 * n}\n", "".join(f"1 {i}\n" for i in range(n)), "\n",
             f"POINT_DATA {n}\n"]
    nc = len(species) if chem is not None else 0
    nfields = 7 + nc + (len(species) if index > 0 else 0)
    parts.append(f"FIELD FieldData {nfields}\n")
    parts += [f"id 1 {n} int\n", _rows(range(n), 9, "%u "), "\n"]
    parts += [f"type 1 {n} int\n", _rows(types, 9, "%u "), "\n"]
    parts += [f"v 3 {n} double\n", _vec_rows(v, "%f"), "\n"]
    parts += [f"rho 1 {n} double\n", _rows(rho, 9, "%f "), "\n"]
    parts += [f"mass 1 {n} double\n", _rows(mass, 9, "%f "), "\n"]
    parts += [f"bvf_phi 1 {n} double\n", _rows(bvf_phi, 9, "%f "), "\n"]
    parts += [f"nu 1 {n} double\n", _rows(nu, 9, "%f "), "\n"]
    if chem is not None:
        for s, name in enumerate(species):
            parts += [f"C[{name}] 1 {n} double\n", _rows(chem[:, s], 9, "%f "), "\n"]
    for s, name in enumerate(species):
        parts += [f"D[{name}] 1 {n} int\n", _rows(counts[:, s], 9, "%u "), "\n"]
    return "".join(parts)


def write_outputs(directory, points, types, mass, rho, nu, species, counts, v=None,
                  bvf_phi=None, bbox=None, chem=None):
    """Write output0.vtk ... output{T-1}.vtk (and output0_boundingBox.vtk
    when ``bbox`` = (xlo, xhi, ylo, yhi, zlo, zhi) is given).

    counts: [T, N, S]; points/v: [N,3] or [T,N,3]; rho: [N] or [T,N].
    """
    os.makedirs(directory, exist_ok=True)
    T = counts.shape[0]
    n = counts.shape[1]
    points = np.asarray(points, np.float64)
    v = np.zeros((n, 3)) if v is None else np.asarray(v, np.float64)
    bvf_phi = np.zeros(n) if bvf_phi is None else np.asarray(bvf_phi, np.float64)
    rho = np.asarray(rho, np.float64)
    if bbox is not None:
        with open(os.path.join(directory, "output0_boundingBox.vtk"), "w") as f:
            f.write("# vtk DataFile Version 4.1\nGenerated by ssa_sdpd\nASCII\n"
                    "DATASET RECTILINEAR_GRID\nDIMENSIONS 2 2 2\n"
                    f"X_COORDINATES 2 double\n{bbox[0]:f} {bbox[1]:f}\n"
                    f"Y_COORDINATES 2 double\n{bbox[2]:f} {bbox[3]:f}\n"
                    f"Z_COORDINATES 2 double\n{bbox[4]:f} {bbox[5]:f}\n")
    paths = []
    for k in range(T):
        pk = points[k] if points.ndim == 3 else points
        vk = v[k] if v.ndim == 3 else v
        rk = rho[k] if rho.ndim == 2 else rho
        text = format_step(pk, types, vk, rk, mass, bvf_phi, nu, species, counts[k], k,
                           None if chem is None else chem[k])
        path = os.path.join(directory, f"output{k}.vtk")
        with open(path, "w") as f:
            f.write(text)
        paths.append(path)
    return paths


def read_step(path):
    """Minimal reader of the files written above: (points [N,3], arrays dict)."""
    with open(path) as f:
        lines = f.read().split("\n")
    n = int(lines[4].split()[1])
    vals, i = [], 5
    while len(vals) < 3 * n:
        vals += [float(x) for x in lines[i].split()]
        i += 1
    points = np.array(vals[:3 * n]).reshape(n, 3)
    while not lines[i].startswith("FIELD"):
        i += 1
    i += 1
    arrays = {}
    while i < len(lines):
        if not lines[i].strip():
            i += 1
            continue
        name, comps, count, dtype = lines[i].split()
        comps, count = int(comps), int(count)
        i += 1
        vals = []
        while len(vals) < comps * count:
            vals += lines[i].split()
            i += 1
        a = np.array(vals[:comps * count], dtype=np.int64 if dtype == "int" else np.float64)
        arrays[name] = a.reshape(count, comps) if comps > 1 else a
    return points, arrays
