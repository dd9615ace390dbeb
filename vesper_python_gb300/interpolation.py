"""Command-line mirror of the reference's interpolation.py: fill the holes of a
probability map sampled on every other voxel (interpolate,
interpolation_functions.py:6-135) on the GPU.

  python -m vesper_python_gb300.interpolation insert -f MAP.npy -s NAME
  python -m vesper_python_gb300.interpolation graph -f MAP.npy -s NAME -m DENSITY.mrc

``insert`` prints what the reference prints (usage banner, the four array
dimensions, the saved name) and writes NAME.npy.  ``graph`` also writes one
MRC map per channel (NAME_0.mrc .. NAME_3.mrc) on the density map's origin
and cell, with the reference's copy of arr[i][j][k][c] for i < nx-2, j < ny-2,
k < nz-2 (conv_prediction_to_mrc, interpolation_functions.py:137-180); the
mrcfile header dumps the reference prints there are not reproduced.
"""
from __future__ import annotations

import argparse

import numpy as np

from . import mrc
from . import vesper as vg


def conv_prediction_to_mrc(arr, reffile, keyidx, outmapfile):
    """One channel of ``arr`` [X][Y][Z][C] as an MRC map (z slowest on disk)
    on the origin and voxel size of ``reffile``."""
    ref = mrc.read_mrc(reffile)
    nx, ny, nz = arr.shape[:3]
    out = np.zeros((nz, ny, nx), np.float32)
    out[:nz - 2, :ny - 2, :nx - 2] = np.transpose(arr[:nx - 2, :ny - 2, :nz - 2, keyidx], (2, 1, 0))
    print(nx, ny, nz)
    mrc.write_mrc(outmapfile, out, voxel_size=float(ref.voxel_size[0]), origin=tuple(float(v) for v in ref.origin))


def main(argv=None):
    print('Usage Modes:\n')
    print('1- Insert: only interpolates the map given.')
    print('2- Graph: interpolates the map given and saves each secondary structure prediction map individually.')
    parser = argparse.ArgumentParser()
    sub = parser.add_subparsers(dest='command')
    insert = sub.add_parser('insert')
    graph = sub.add_parser('graph')
    insert.add_argument('-f', type=str, required=True, help='Map array (.npy)')
    insert.add_argument('-s', type=str, required=True, help='Name for new map to be saved (string)')
    graph.add_argument('-f', type=str, required=True, help='Map array (.npy)')
    graph.add_argument('-s', type=str, required=True, help='Name for individual maps (string)')
    graph.add_argument('-m', type=str, required=True,
                       help='Name of density map file. NOTE: VOXEL SPACIING MUST BE 1. (.mrc)')
    args = parser.parse_args(argv)
    if args.command not in ('insert', 'graph'):
        return
    orig_data = np.load(args.f)
    np.set_printoptions(precision=3)
    for a in range(4):
        print(orig_data.shape[a])
    vg.interpolate(orig_data)
    np.save(args.s, orig_data)
    print('Saved interpolated map as: ' + args.s + '.npy')
    if args.command == 'graph':
        for i in range(4):
            conv_prediction_to_mrc(orig_data, args.m, i, args.s + f"_{i}.mrc")


if __name__ == '__main__':
    main()
