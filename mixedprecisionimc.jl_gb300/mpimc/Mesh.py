"""Mesh generation: the reference's ``Mesh`` module (src/imc_mesh.jl:10-259).

``mesh_generation(inputs)`` returns a :class:`MeshStruct` with the reference's
29 fields.  Input values are rounded to the deck precision exactly where the
reference parses them in that precision, and held as float64; mesh nodes of
non-uniform meshes stay float64 (src/imc_input.jl:91-92).  2D arrays have
shape (Nx, Ny) like the Julia arrays, and flatten x-fastest (Fortran order)
into the engine's cell index ix + iy*Nx.
"""
from dataclasses import dataclass, field
from typing import Any

import numpy as np

from .Utilities import tointeger


def _p(precision, v):
    """Julia parse(precision, s) / convert(precision, x), held as float64."""
    return float(precision(float(v)))


def linrange(a, b, n, precision):
    """Julia LinRange{precision}(a, b, n): element j is T((1-t)*a + t*b), t = j/(n-1)."""
    d = n - 1
    out = np.empty(n)
    for j in range(n):
        t = j / d if d > 0 else 0.0
        out[j] = _p(precision, (1.0 - t) * a + t * b)
    return out


@dataclass
class MeshStruct:
    """src/imc_mesh.jl:10-40, field for field."""
    temp: Any
    temp_surf: Any
    fleck: Any
    beta: Any
    sigma: Any
    sigma_a: Any
    sigma_s: Any
    energydep: Any
    emittedenergy: Any
    totalenergy: float
    totalenergydep: float
    lostenergy: float
    radenergyold: float
    bee: Any
    radsource: Any
    radenergydens: Any
    matenergydens: Any
    temp_saved: list
    energyincrease_saved: list
    radenergy_saved: list
    matenergy_saved: list
    energyscales: Any
    distancescale: float
    centers: Any
    nodes: Any
    dx: Any
    dy: Any
    perimeter: Any
    Ncells: Any
    engine: Any = field(default=None, repr=False)


def _count(q, what):
    """tointeger(xsize/dx): the reference raises InexactError unless integral."""
    n = int(round(q))
    if abs(q - n) > 1e-6 * max(1.0, abs(q)):
        raise ValueError("%s = %r is not an integer number of cells" % (what, q))
    return n


def region_joiner(geometry, regions, values, nodes, Ncells, precision):
    """src/imc_mesh.jl:175-220: per-cell values from region boundaries."""
    if geometry == "1D":
        N = Ncells
        regions = list(regions) if not isinstance(regions, str) else [regions]
        if len(regions) <= 1:
            return np.full(N, _p(precision, values[0]))
        out = np.zeros(N)
        ri = 0
        for i in range(N):
            if float(regions[ri]) >= nodes[i + 1]:
                out[i] = _p(precision, values[ri])
            else:
                ri += 1
                out[i] = _p(precision, values[ri])
        return out
    nx, ny = Ncells
    reg = regions[0]
    if isinstance(reg, str) or np.ndim(reg) == 0 or len(reg) <= 1:
        return np.full((nx, ny), _p(precision, values[0]))
    # a single region written as ((x0, x1), (y0, y1)) is taken as one region
    if len(reg) == 2 and np.ndim(reg[0]) == 1 and np.ndim(reg[0][0]) == 0:
        reg = (reg,)
    out = np.zeros((nx, ny))
    xn, yn = np.asarray(nodes[0]), np.asarray(nodes[1])
    for r, ((xs, xe), (ys, ye)) in enumerate(reg):
        xsi = int(np.nonzero(xn <= xs)[0][-1])
        xei = int(np.nonzero(xn <= xe)[0][-1])
        ysi = int(np.nonzero(yn <= ys)[0][-1])
        yei = int(np.nonzero(yn <= ye)[0][-1])
        out[xsi:xei, ysi:yei] = _p(precision, values[r])
    return out


def surface_definer(geometry, regions, values, perimeter, nodes, Ncells, precision):
    """src/imc_mesh.jl:222-259: surface temperatures (1D pair; 2D four faces)."""
    if geometry == "1D":
        return (_p(precision, values[0]), _p(precision, values[1]))
    vals = values[0]
    regs = regions[0]
    faces = []
    for i in range(4):
        v = vals[i]
        sv = [v] if np.ndim(v) == 0 else list(v)
        r = regs[i]
        rr = [r] if np.ndim(r) == 0 else list(r)
        if i < 2:
            faces.append(region_joiner("1D", rr, sv, nodes[0], Ncells[0], precision))
        else:
            faces.append(region_joiner("1D", rr, sv, nodes[1], Ncells[1], precision))
    return faces


def mesh_generation(inputs):
    """src/imc_mesh.jl:42-173."""
    geometry = str(inputs["GEOMETRY"]).upper()
    meshtype = str(inputs["MESHTYPE"]).upper()
    precision = inputs.get("PRECISION", np.float64)
    if geometry == "1D":
        if meshtype == "UNIFORM":
            xsize = _p(precision, inputs["XSIZE"])
            dxt = _p(precision, inputs["DX"])
            N = _count(float(precision(xsize) / precision(dxt)), "XSIZE/DX")
            dx = np.full(N, dxt)
            dy = 1.0
            nodes = linrange(0.0, xsize, N + 1, precision)
            centers = linrange(dxt / 2, xsize - dxt / 2, N, precision)
        elif meshtype == "NONUNIFORM":
            nn = np.asarray(inputs["MESHNODES"], dtype=np.float64)
            centers = np.array([_p(precision, v) for v in (nn[:-1] + nn[1:]) / 2])
            dx = np.array([_p(precision, v) for v in (nn[1:] - nn[:-1])])
            dy = 1.0
            nodes = np.array([_p(precision, v) for v in nn])
            N = len(dx)
        else:
            raise ValueError("MESHTYPE must be UNIFORM or NONUNIFORM")
        Ncells = N
        perimeter = (0.0, 0.0)
        shape = (N,)
    elif geometry == "2D":
        if meshtype == "UNIFORM":
            xsize = _p(precision, inputs["XSIZE"])
            ysize = _p(precision, inputs["YSIZE"])
            dxt = _p(precision, inputs["DX"])
            dyt = _p(precision, inputs["DY"])
            # the reference divides YSIZE by DX here (src/imc_mesh.jl:86)
            Ncells = (_count(float(precision(xsize) / precision(dxt)), "XSIZE/DX"),
                      _count(float(precision(ysize) / precision(dxt)), "YSIZE/DX"))
            dx = np.full(Ncells[0], dxt)
            dy = np.full(Ncells[1], dyt)
            xnodes = linrange(0.0, xsize, Ncells[0] + 1, precision)
            ynodes = linrange(0.0, ysize, Ncells[1] + 1, precision)
            centers = (linrange(dxt / 2, xsize - dxt / 2, Ncells[0], precision),
                       linrange(dyt / 2, ysize - dyt / 2, Ncells[1], precision))
            nodes = (xnodes, ynodes)
        elif meshtype == "NONUNIFORM":
            xn = np.asarray(inputs["XMESHNODES"], dtype=np.float64)
            yn = np.asarray(inputs["YMESHNODES"], dtype=np.float64)
            centers = (np.array([_p(precision, v) for v in (xn[:-1] + xn[1:]) / 2]),
                       np.array([_p(precision, v) for v in (yn[:-1] + yn[1:]) / 2]))
            dx = np.array([_p(precision, v) for v in (xn[1:] - xn[:-1])])
            dy = np.array([_p(precision, v) for v in (yn[1:] - yn[:-1])])
            nodes = (np.array([_p(precision, v) for v in xn]), np.array([_p(precision, v) for v in yn]))
            Ncells = (len(dx), len(dy))
        else:
            raise ValueError("MESHTYPE must be UNIFORM or NONUNIFORM")
        perimeter = tuple(np.zeros(n) for n in (Ncells[0], Ncells[0], Ncells[1], Ncells[1]))
        shape = Ncells
    else:
        raise ValueError("GEOMETRY must be 1D or 2D")

    T_init = _p(precision, inputs["T_INIT"])
    T_surface = surface_definer(geometry, inputs.get("T_SURFACE_REGS", [""]), inputs["T_SURFACE_VALS"], perimeter,
                                nodes, Ncells, precision)
    temp = np.full(shape, T_init)
    fleck = np.zeros(shape)
    beta = np.ones(shape)
    sa = region_joiner(geometry, inputs["SIGMA_A_REGS"], inputs["SIGMA_A_VALS"], nodes, Ncells, precision)
    sap = region_joiner(geometry, inputs["SIGMA_A_REGS"], inputs["SIGMA_A_POWERS"], nodes, Ncells, precision)
    ss = region_joiner(geometry, inputs["SIGMA_S_REGS"], inputs["SIGMA_S_VALS"], nodes, Ncells, precision)
    ssp = region_joiner(geometry, inputs["SIGMA_S_REGS"], inputs["SIGMA_S_POWERS"], nodes, Ncells, precision)
    es = inputs["ENERGYSCALES"]
    if len(es) == 1 and isinstance(es[0], str):
        energyscales = np.array([_p(precision, es[0])])
    else:
        energyscales = np.array(sorted([_p(precision, v) for v in es], reverse=True))
    distancescale = _p(precision, inputs["DISTANCESCALE"])
    sa = np.array([_p(precision, v) for v in (sa / distancescale).ravel()]).reshape(shape)
    ss = np.array([_p(precision, v) for v in (ss / distancescale).ravel()]).reshape(shape)
    sigma_a = np.stack([sa, sa, sap], axis=-1)
    sigma_s = np.stack([ss, ss, ssp], axis=-1)
    sigma = sigma_a + sigma_s
    radsource = region_joiner(geometry, inputs["RADSOURCE_REGS"], inputs["RADSOURCE_VALS"], nodes, Ncells, precision)
    K = len(energyscales)
    energydep = np.zeros(shape + (K,))
    emittedenergy = np.zeros(shape + (K,))
    bee = region_joiner(geometry, inputs["BEE_REGS"], inputs["BEE_VALS"], nodes, Ncells, precision)
    return MeshStruct(
        temp=temp, temp_surf=T_surface, fleck=fleck, beta=beta, sigma=sigma, sigma_a=sigma_a, sigma_s=sigma_s,
        energydep=energydep, emittedenergy=emittedenergy, totalenergy=0.0, totalenergydep=0.0, lostenergy=0.0,
        radenergyold=0.0, bee=bee, radsource=radsource, radenergydens=np.zeros(shape),
        matenergydens=np.zeros(shape), temp_saved=[temp.copy()], energyincrease_saved=[], radenergy_saved=[],
        matenergy_saved=[], energyscales=energyscales, distancescale=distancescale, centers=centers, nodes=nodes,
        dx=dx, dy=dy, perimeter=perimeter, Ncells=Ncells)
