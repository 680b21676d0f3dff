"""Host driver of a smoothing pass over a whole tet mesh (VertexSmoother::smooth,
VertexSmoother.cpp:19-46: smoothSingle over the interior vertices, then
smoothSurface over the surface vertices).

The reference visits the vertices one by one, each seeing the moves made
before it.  Here the vertices are grouped by a colouring in which no two
vertices of a tet share a colour, so the stars of one colour are independent
and run as one batch (``tw_smooth_stars``); the colours run in order, each
seeing the moves of the previous ones.  Each star lists the centre's tets in
ascending tet order (the reference iterates an unordered set).  Box corners
(kind 3) are locked and skipped, as ``is_on_bbox`` vertices are (:121).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .synthetic import greedy_colouring, vertex_stars

KIND_INTERIOR = 0
KIND_SURFACE = 1
KIND_BOUNDARY = 2
KIND_LOCKED = 3


@dataclass
class PassLog:
    """What one pass did: one record per batch (phase, colour, centres, status, positions)."""
    batches: list = field(default_factory=list)

    @property
    def stars(self) -> int:
        return sum(len(b["centers"]) for b in self.batches)

    def status_counts(self) -> np.ndarray:
        if not self.batches:
            return np.zeros(6, np.int64)
        return np.bincount(np.concatenate([b["status"] for b in self.batches]).astype(np.int64),
                           minlength=6)


def star_batch_of(centers: np.ndarray, tets: np.ndarray, face_flags: np.ndarray, off, ids):
    """CSR star batch (star_off, star tets, star face flags) of the given centres."""
    counts = (off[centers + 1] - off[centers]).astype(np.int64)
    star_off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    sel = np.concatenate([ids[off[c]:off[c + 1]] for c in centers]) if len(centers) else \
        np.zeros(0, np.int32)
    return star_off, tets[sel], face_flags[sel]


def smoothing_pass(xyz: np.ndarray, tets: np.ndarray, face_flags: np.ndarray, kind: np.ndarray,
                   run_batch, colour: np.ndarray | None = None) -> tuple[np.ndarray, PassLog]:
    """One pass: interior vertices colour by colour, then surface (and boundary) vertices.

    ``run_batch(xyz, star_off, star_tets, centers, star_face_flags, star_kinds)`` evaluates one
    batch on the current positions and returns (positions [n,3], status [n]); it is
    ``Context.smooth_stars`` (after pushing moved vertices with ``mesh_update_vertices``) on the
    device, or the oracle in the tests.  Returns the new positions and the log.
    """
    xyz = np.array(xyz, dtype=np.float64, copy=True)
    nv = len(xyz)
    if colour is None:
        colour = greedy_colouring(tets, nv)
    off, ids = vertex_stars(tets, nv)
    log = PassLog()
    for phase, kinds_in in (("single", (KIND_INTERIOR,)), ("surface", (KIND_SURFACE, KIND_BOUNDARY))):
        for c in range(int(colour.max()) + 1):
            centers = np.nonzero((colour == c) & np.isin(kind, kinds_in) &
                                 (off[1:] > off[:-1]))[0].astype(np.int32)
            if len(centers) == 0:
                continue
            star_off, star_tets, star_ff = star_batch_of(centers, tets, face_flags, off, ids)
            sk = kind[centers].astype(np.uint8)
            pos, st = run_batch(xyz, star_off, star_tets, centers, star_ff, sk)
            moved = st == 2
            xyz[centers[moved]] = pos[moved]
            log.batches.append({"phase": phase, "colour": c, "centers": centers,
                                "status": np.asarray(st).copy(), "pos": np.asarray(pos).copy()})
    return xyz, log


def device_runner(ctx):
    """run_batch for ``smoothing_pass`` on a device context whose resident mesh holds the pass's
    starting positions; each batch's moves are pushed to the resident mesh at once, so it
    always equals the pass's current positions."""

    def run(xyz, star_off, star_tets, centers, star_ff, star_kinds):
        pos, st = ctx.smooth_stars(star_off, star_tets, centers, star_ff, star_kinds)
        moved = st == 2
        if moved.any():
            ctx.mesh_update_vertices(centers[moved], pos[moved])
        return pos, st

    return run
