"""Algorithmic work per unit of the force path: the fixed constants the rooflines divide by
the measured time. They count the work of the algorithm, not what a kernel executes.

Pairs (src/frclong.c:56-218 with src/ljfrc.c:21-71 and src/elecfrc.c:17-60): a pair is one
inter-molecular site pair (i, j) with r^2 < rc^2, counted once (Newton's third law).
  - LJ pair: difference 3, minimum image 6, r^2 5, 1/r^2 1, s^6 3, s^12 1, energy 2, F/r 2,
    force accumulation 6: 29 FP32 FLOP;
  - Ewald real space or Wolf pair alone: difference, image and r^2 14, erfc 12, energy 4,
    F/r 6, accumulation 6: 42 FLOP (the rsqrt and exp are special-function operations);
  - LJ + electrostatics, sharing the distance and the accumulation: 55 FLOP.
Reciprocal space (src/frclong.c:988-1048), per (half-space k-vector, site): 10 FLOP in the
structure-factor pass (phase 5, accumulation of Re and Im), 12 in the force pass.
Bytes:
  - neighbour streaming of the pair stage, per entry of the half list: its 4 B j-cluster
    index, its 16 B periodic shift and the j-cluster's 8 slots of 32 B (position row and
    charge/LJ row); per site its 16 B position and 24 B of fixed-point force;
  - list build, per entry of the full list: 4 B index, 16 B shift, 4 B image; per site its
    FP64 position read, wrapped position and binned copy (3 x 3 x 8 B);
  - the tricubic solid-fluid gather: 64 FP32 table values (256 B) per site.
"""

FLOP_PAIR_LJ = 29.0
FLOP_PAIR_ELEC = 42.0
FLOP_PAIR = 55.0
FLOP_K_S = 10.0
FLOP_K_F = 12.0

# FLOP the FP32 table passes execute, per site: S(k) 4 FMAs per (row, |kz|) for both signs of
# kz plus q X^kx Y^ky per row; forces 8 FMAs per (row, |kz|) plus the per-row epilogue
FLOP_SK_ROWKZ, FLOP_SK_ROW = 8.0, 8.0
FLOP_KF_ROWKZ, FLOP_KF_ROW = 16.0, 18.0

SF_BYTES_PER_SITE = 256.0


def neighbour_streaming_bytes(full_entries: int, sites: int) -> float:
    """Bytes the pair stage streams for a full cluster-pair list of full_entries entries
    (half of them are evaluated) over sites sites."""
    half = 0.5 * full_entries
    return full_entries * 20.0 + half * 8 * 32.0 + sites * 40.0


def list_build_bytes(full_entries: int, sites: int) -> float:
    """Bytes the list build writes and reads."""
    return full_entries * 24.0 + sites * 3 * 8.0 * 3
