"""Nastran bulk-data (BDF) reader for the element types of the GPU path.

Reads the cards a shell or solid model of this path needs -- GRID (with
CORD2R rectangular coordinate systems), CQUAD4, CHEXA, SPC1 and FORCE --
in small-field, large-field (``*``) and free-field (comma) formats with
continuation lines, and returns a problem record for
:class:`tacs_gb300.problem.GpuModel`.  The numbering follows the
reference's mesh loader (src/io/TACSMeshLoader.cpp): nodes in increasing
GRID id, elements in card order, CQUAD4 nodes 1-2-4-3 (the tensor-product
order of TACSShellQuadBasis<2>), CHEXA nodes 1-2-4-3-5-6-8-7
(TACSLinearHexaBasis).  Materials, thicknesses and loads other than FORCE
are given by the caller, as pyTACS element call-backs do.
"""
from __future__ import annotations

import re

import numpy as np

from . import meshes


def _real(s):
    """Nastran real: 1.5, -.5, 1.07+7, 2.5906-4, 1.E-5, 3."""
    s = s.strip()
    if not s:
        return 0.0
    try:
        return float(s)
    except ValueError:
        pass
    body = s.replace("D", "E").replace("d", "E")
    for i in range(len(body) - 1, 0, -1):
        if body[i] in "+-" and body[i - 1] not in "eE":
            return float(body[:i] + "E" + body[i:])
    return float(body)


def _int(s, default=0):
    s = s.strip()
    return int(s) if s else default


def _cards(lines):
    """Yield (name, fields) with continuations merged; fields exclude the
    name and continuation markers."""
    card = None
    for raw in lines:
        line = raw.rstrip("\n")
        if not line.strip() or line.lstrip().startswith("$"):
            continue
        if "$" in line:
            line = line[:line.index("$")]
        if "," in line:
            parts = [p.strip() for p in line.split(",")]
            head = parts[0]
            if head.startswith("+") or head.startswith("*") or head == "":
                if card is not None:
                    card[1].extend(parts[1:])
                continue
            if card is not None:
                yield card
            card = (head.upper().rstrip("*"), parts[1:])
            continue
        head = line[:8].strip()
        if head.startswith("+") or head.startswith("*") or head == "":
            # continuation: 16-character fields after a large-field marker
            # ("*..."), 8-character ones otherwise; columns 9-72 either way
            if card is not None:
                width = 16 if head.startswith("*") else 8
                body = line[8:72]
                card[1].extend(body[k:k + width]
                               for k in range(0, len(body), width))
            continue
        large = head.endswith("*")
        width = 16 if large else 8
        if card is not None:
            yield card
        body = line[8:72]
        card = (head.upper().rstrip("*"),
                [body[k:k + width] for k in range(0, len(body), width)])
    if card is not None:
        yield card


def _cord2r(f):
    """Basic-frame origin and rotation of a CORD2R (A origin, B on the z
    axis, C in the xz plane)."""
    a = np.array([_real(x) for x in f[2:5]])
    b = np.array([_real(x) for x in f[5:8]])
    c = np.array([_real(x) for x in f[8:11]])
    ez = (b - a) / np.linalg.norm(b - a)
    ey = np.cross(ez, c - a)
    ey /= np.linalg.norm(ey)
    ex = np.cross(ey, ez)
    return a, np.stack([ex, ey, ez], axis=1)


def read_bdf(path, thickness=1.0, E=70e9, nu=0.3, rho=2700.0, ys=2.7e8):
    """Problem record of a BDF file (one element type: all CQUAD4 or all
    CHEXA), one design variable per element with thickness (or the solid
    scale) ``thickness``.  Extra keys: ``grid_ids`` (GRID id of each node),
    ``elem_ids`` (element id of each element)."""
    with open(path) as fh:
        lines = fh.readlines()
    cards = list(_cards(lines))
    # component names from property comments ("$ ... Property 1 : PLATE")
    names = {}
    for line in lines:
        m = re.match(r"\s*\$.*Property\s+(\d+)\s*:\s*(.*\S)", line)
        if m:
            names[int(m.group(1))] = m.group(2)
    cords, grids, quads, hexes, spcs, forces = {}, {}, [], [], [], []
    pids = []
    for name, f in cards:
        if name == "CORD2R":
            cords[_int(f[0])] = _cord2r(f)
        elif name == "GRID":
            gid, cp = _int(f[0]), _int(f[1])
            x = np.array([_real(v) for v in f[2:5]])
            grids[gid] = (cp, x)
        elif name == "CQUAD4":
            quads.append((_int(f[0]), [_int(v) for v in f[2:6]]))
            pids.append(_int(f[1]))
        elif name == "CHEXA":
            hexes.append((_int(f[0]), [_int(v) for v in f[2:10]]))
            pids.append(_int(f[1]))
        elif name == "SPC1":
            comps = f[1].strip()
            ids = [_int(v) for v in f[2:] if v.strip()]
            if len(f) > 4 and f[3].strip().upper() == "THRU":
                ids = list(range(_int(f[2]), _int(f[4]) + 1))
            spcs.append((comps, ids))
        elif name == "FORCE":
            gid = _int(f[1])
            mag = _real(f[3])
            vec = np.array([_real(v) for v in f[4:7]])
            forces.append((gid, mag * vec))
    if quads and hexes:
        raise ValueError("one element type per model")
    ids = sorted(grids)
    index = {g: k for k, g in enumerate(ids)}
    xyz = np.zeros((len(ids), 3))
    for g, (cp, x) in grids.items():
        if cp:
            if cp not in cords:
                raise NotImplementedError(f"coordinate system {cp} (only "
                                          "CORD2R is read)")
            o, R = cords[cp]
            x = o + R @ x
        xyz[index[g]] = x
    if quads:
        conn = np.array([[index[n[0]], index[n[1]], index[n[3]], index[n[2]]]
                         for _, n in quads], np.int32)
        et, vpn, eids = meshes.SHELL, 6, [e for e, _ in quads]
    else:
        conn = np.array([[index[n[k]] for k in (0, 1, 3, 2, 4, 5, 7, 6)]
                         for _, n in hexes], np.int32)
        et, vpn, eids = meshes.HEX, 3, [e for e, _ in hexes]
    ne = len(conn)
    p = meshes._base(et, xyz, conn, np.full(ne, float(thickness)),
                     np.arange(ne), (rho, E, nu, ys))
    masks = {}
    for comps, gids in spcs:
        m = 0
        for ch in comps:
            if ch.isdigit() and 1 <= int(ch) <= vpn:
                m |= 1 << (int(ch) - 1)
        for g in gids:
            masks[index[g]] = masks.get(index[g], 0) | m
    nodes = sorted(masks)
    p["bc_nodes"] = np.array(nodes, np.int32)
    p["bc_masks"] = np.array([masks[n] for n in nodes], np.int32)
    force = np.zeros((len(ids), vpn))
    for g, v in forces:
        force[index[g], :3] += v
    p["force"] = force.ravel()
    p["grid_ids"] = np.array(ids)
    p["elem_ids"] = np.array(eids)
    p["elem_pids"] = np.array(pids, np.int32)
    p["pid_names"] = {pid: names.get(pid, "") for pid in sorted(set(pids))}
    return p


def write_bdf(path, p, pid_names=None):
    """Free-field BDF of a problem record's GRIDs (basic frame, full
    precision), CQUAD4 / CHEXA elements (property ids from ``elem_pids``,
    default 1) and SPC1 cards, readable by read_bdf (ids: node index + 1,
    element index + 1)."""
    xyz = np.asarray(p["xpts"]).reshape(-1, 3)
    shell = int(p["elem_type"]) == meshes.SHELL
    npe = 4 if shell else 8
    conn = np.asarray(p["conn"]).reshape(-1, npe)
    pids = np.asarray(p.get("elem_pids", np.ones(len(conn), np.int32)))
    order = (0, 1, 3, 2) if shell else (0, 1, 3, 2, 4, 5, 7, 6)
    out = ["BEGIN BULK"]
    for pid in sorted(set(int(x) for x in pids)):
        nm = (pid_names or {}).get(pid, f"COMP{pid}")
        out.append(f"$ Property {pid} : {nm}")
        out.append(f"{'PSHELL' if shell else 'PSOLID'},{pid},1")
    for k, x in enumerate(xyz):
        out.append(f"GRID,{k + 1},0,{float(x[0])!r},{float(x[1])!r},{float(x[2])!r}")
    name = "CQUAD4" if shell else "CHEXA"
    for e, nodes in enumerate(conn):
        ns = ",".join(str(int(nodes[q]) + 1) for q in order)
        out.append(f"{name},{e + 1},{int(pids[e])},{ns}")
    for node, mask in zip(p["bc_nodes"], p["bc_masks"]):
        comps = "".join(str(k + 1) for k in range(6) if (int(mask) >> k) & 1)
        out.append(f"SPC1,1,{comps},{int(node) + 1}")
    out.append("ENDDATA")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")
