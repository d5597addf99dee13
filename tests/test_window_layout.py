"""Shared-memory layout of the tile kernel (k_tiles32), checked on the CPU
from the constants in its source.

A tile holds ECS_TILE_X x ECS_TILE_Y x ECS_TILE_Z = 32 cells.  With the ions
sorted, lane L of a warp starts on the ions of the tile's L-th cell, so:

- the deposit window and the z numerators (one 4-byte word a node at strides
  kSY, kSZ) put the 32 cells' base nodes in 32 different banks;
- the x, y numerators (a float2 a node at strides kEX, kEXY) are read 16
  lanes at a time, and each z plane's 16 cells land in 16 different float2
  bank pairs;
- every node a window ion touches (its cell's 8 corners, the cell within one
  cell of the tile) lies inside the arrays.
"""
import re
from pathlib import Path

CSRC = Path(__file__).resolve().parents[1] / "ecsprt_gb300" / "csrc"


def _consts():
    hdr = (CSRC / "ecs_internal.cuh").read_text()
    src = (CSRC / "ecs_particles.cu").read_text()
    t = {a: int(re.search(rf"#define ECS_TILE_{a} (\d+)", hdr).group(1)) for a in "XYZ"}
    kex = int(re.search(r"constexpr int kEX = (\d+), kEXY = kEX \* kWY;", src).group(1))
    m = re.search(r"constexpr int kSY = (\d+), kSZ = (\d+);", src)
    ksy, ksz = int(m.group(1)), int(m.group(2))
    # declarations the layout below assumes
    assert "__shared__ float2 ewxy[kEXY * kWZ];" in src
    assert "__shared__ float ewz[kWPad];" in src
    assert "__shared__ unsigned win[5][kWPad];" in src
    assert "constexpr int kWPad = kSZ * kWZ;" in src
    return t, kex, ksy, ksz


def test_tile_cells_map_to_distinct_banks():
    t, kex, ksy, ksz = _consts()
    cells = [(x, y, z) for z in range(t["Z"]) for y in range(t["Y"]) for x in range(t["X"])]
    assert len(cells) == 32
    # 4-byte words (deposit window, z numerators): one bank each
    assert len({(x + ksy * y + ksz * z) % 32 for x, y, z in cells}) == 32
    # 8-byte float2 (x, y numerators): half-warps of 16 lanes, one z plane each
    for z in range(t["Z"]):
        plane = [(x + kex * y) % 16 for x, y, zz in cells if zz == z]
        assert len(plane) == 16 and len(set(plane)) == 16


def test_window_accesses_stay_inside_the_arrays():
    t, kex, ksy, ksz = _consts()
    wx, wy, wz = t["X"] + 3, t["Y"] + 3, t["Z"] + 3  # window nodes per axis
    cx, cy, cz = t["X"] + 2, t["Y"] + 2, t["Z"] + 2  # window cells per axis
    kexy = kex * wy
    wpad = ksz * wz
    assert wx <= kex and wx <= ksy and wy * ksy <= ksz
    # the fill writes every window node once, at distinct places
    xy = {gz * kexy + gy * kex + gx for gz in range(wz) for gy in range(wy) for gx in range(wx)}
    zw = {gz * ksz + gy * ksy + gx for gz in range(wz) for gy in range(wy) for gx in range(wx)}
    assert len(xy) == len(zw) == wx * wy * wz
    assert max(xy) < kexy * wz and max(zw) < wpad
    # an ion of window cell (i, j, k) reads and deposits at its 8 corners
    for k in range(cz):
        for j in range(cy):
            for i in range(cx):
                for b in range(8):
                    dx, dy, dz = b & 1, (b >> 1) & 1, b >> 2
                    assert (k + dz) * kexy + (j + dy) * kex + (i + dx) in xy
                    assert (k + dz) * ksz + (j + dy) * ksy + (i + dx) in zw
