"""Command line of the GB300 VESPER path: the same ``orig`` / ``prob``
sub-commands, flags, defaults and stdout as the reference's ``main.py``
(main.py:68-370), e.g.

    python -m vesper_python_gb300.main orig -a MAP1.mrc -b MAP2.mrc -t 0.1 -T 0.1 -s 7 -A 30
    python -m vesper_python_gb300.main prob -a MAP1.mrc -npa P1.npy -b MAP2.mrc -npb P2.npy

Quirks kept from the reference: ``-S``/``-E`` are ``type=bool`` (any non-empty
string is True), ``-t``/``-T`` default to 0.0, ``-A`` is a float, ``-P`` is
accepted but unused, the prob statistics default to -10 ("compute").
"""
from __future__ import annotations

import argparse

import numpy as np

from .vesper import fastVEC, mrc_obj, mrc_set_vox_size, search_map_fft, search_map_fft_prob

MODE_NAMES = {"V": "VecProduct", "O": "Overlap", "C": "CC", "P": "PCC", "L": "Laplacian"}


def build_parser():
    parser = argparse.ArgumentParser()
    subparser = parser.add_subparsers(dest="command")
    orig = subparser.add_parser("orig")
    prob = subparser.add_parser("prob")
    mode_help = ("V: vector product mode (default)\nO: overlap mode\nC: Cross Correlation Coefficient Mode\n"
                 "P: Pearson Correlation Coefficient Mode\nL: Laplacian Filtering Mode")
    orig.add_argument("-a", type=str, required=True, help="MAP1.mrc (large)")
    orig.add_argument("-b", type=str, required=True, help="MAP2.mrc (small)")
    orig.add_argument("-t", type=float, help="Threshold of density map1")
    orig.add_argument("-T", type=float, help="Threshold of density map2")
    orig.add_argument("-g", type=float, default=16.0,
                      help="Bandwidth of the Gaussian filter def=16.0, sigma = 0.5*[value entered]")
    orig.add_argument("-s", type=float, default=7.0, help="Sampling voxel spacing def=7.0")
    orig.add_argument("-A", type=float, default=30.0, help="Sampling angle spacing def=30.0")
    orig.add_argument("-N", type=int, default=10, help="Refine Top [int] models def=10")
    orig.add_argument("-S", type=bool, default=False, help="Show topN models in PDB format def=false")
    orig.add_argument("-M", type=str, default="V", help=mode_help)
    orig.add_argument("-E", type=bool, default=False, help="Evaluation mode of the current position def=false")
    orig.add_argument("-o", type=str, default=None, help="Output folder name")

    prob.add_argument("-a", type=str, required=True, help="MAP1.mrc (large)")
    prob.add_argument("-npa", type=str, required=True, help="numpy array for Predictions for map 1")
    prob.add_argument("-b", type=str, required=True, help="MAP2.mrc (small)")
    prob.add_argument("-npb", type=str, required=True, help="numpy array for Predictions for map 2")
    prob.add_argument("-alpha", type=float, default=0.5, required=False,
                      help="The weighting parameter for alpha mixing def=0.0")
    prob.add_argument("-t", type=float, help="Threshold of density map1")
    prob.add_argument("-T", type=float, help="Threshold of density map2")
    prob.add_argument("-g", type=float, default=16.0,
                      help="Bandwidth of the Gaussian filter def=16.0, sigma = 0.5*[value entered]")
    prob.add_argument("-s", type=float, default=7.0, help="Sampling voxel spacing def=7.0")
    prob.add_argument("-A", type=float, default=30.0, help="Sampling angle spacing def=30.0")
    prob.add_argument("-N", type=int, default=10, help="Refine Top [int] models def=10")
    prob.add_argument("-S", type=bool, default=False, help="Show topN models in PDB format def=false")
    prob.add_argument("-M", type=str, default="V", help=mode_help)
    prob.add_argument("-E", type=bool, default=False, help="Evaluation mode of the current position def=false")
    prob.add_argument("-P", type=int, default=4, help="Number of processors to use def=4")
    prob.add_argument("-vav", type=float, help="Pre-computed average for density map")
    prob.add_argument("-vstd", type=float, help="Pre-computed standard deviation for density map")
    prob.add_argument("-pav", type=float, help="Pre-computed average for probability map")
    prob.add_argument("-pstd", type=float, help="Pre-computed standard deviation for probability map")
    prob.add_argument("-o", type=str, default=None, help="Output folder name")
    return parser


def _unify(mrc_N1, mrc_N2, voxel_spacing):
    """main.py:166-185."""
    if mrc_N1.xdim > mrc_N2.xdim:
        dim = mrc_N2.xdim = mrc_N2.ydim = mrc_N2.zdim = mrc_N1.xdim
        mrc_N2.orig[0] = mrc_N2.cent[0] - 0.5 * voxel_spacing * mrc_N2.xdim
        mrc_N2.orig[1] = mrc_N2.cent[1] - 0.5 * voxel_spacing * mrc_N2.xdim
        mrc_N2.orig[2] = mrc_N2.cent[2] - 0.5 * voxel_spacing * mrc_N2.xdim
    else:
        dim = mrc_N1.xdim = mrc_N1.ydim = mrc_N1.zdim = mrc_N2.xdim
        mrc_N1.orig[0] = mrc_N1.cent[0] - 0.5 * voxel_spacing * mrc_N1.xdim
        mrc_N1.orig[1] = mrc_N1.cent[1] - 0.5 * voxel_spacing * mrc_N1.xdim
        mrc_N1.orig[2] = mrc_N1.cent[2] - 0.5 * voxel_spacing * mrc_N1.xdim
    for m in (mrc_N1, mrc_N2):
        m.dens = np.zeros((dim ** 3, 1))
        m.vec = np.zeros((dim, dim, dim, 3), dtype="float32")
        m.data = np.zeros((dim, dim, dim))
    return dim


def run_orig(mrc1, mrc2, threshold1, threshold2, bandwidth, voxel_spacing, angle_spacing, topN, showPDB, modeVal,
             evalMode, folder, blank_lines=True):
    """main.py:158-206 on already-constructed map objects."""
    mrc1, mrc_N1 = mrc_set_vox_size(mrc1, threshold1, voxel_spacing)
    mrc2, mrc_N2 = mrc_set_vox_size(mrc2, threshold2, voxel_spacing)
    _unify(mrc_N1, mrc_N2, voxel_spacing)
    if blank_lines:
        print()
    mrc_N1 = fastVEC(mrc1, mrc_N1, bandwidth)
    mrc_N2 = fastVEC(mrc2, mrc_N2, bandwidth)
    if blank_lines:
        print()
    modeVal = MODE_NAMES.get(modeVal, modeVal)
    return search_map_fft(mrc_N1, mrc_N2, TopN=topN, ang=angle_spacing, mode=modeVal, is_eval_mode=evalMode,
                          showPDB=showPDB, folder=folder)


def alpha_is_zero(objA, objB, threshold1, threshold2, bandwidth, voxel_spacing, angle_spacing, topN, showPDB,
                  modeVal, evalMode, folder=None):
    """main.py:17-65 (the prob command with alpha == 0): the orig path without
    its two blank lines."""
    return run_orig(mrc_obj(objA), mrc_obj(objB), threshold1, threshold2, bandwidth, voxel_spacing, angle_spacing,
                    topN, showPDB, modeVal, evalMode, folder, blank_lines=False)


def run_prob(objA, objB, npA, npB, threshold1, threshold2, bandwidth, voxel_spacing, angle_spacing, topN, showPDB,
             alpha, vave, vstd, pave, pstd, num_processors, folder, maps=None, prob_arrays=None):
    """main.py:282-370.  ``maps``/``prob_arrays`` let callers pass in-memory
    objects instead of file paths."""
    prob_maps = np.load(npA).astype(np.float32) if prob_arrays is None else prob_arrays[0].astype(np.float32)
    prob_maps_chain = np.load(npB).astype(np.float32) if prob_arrays is None else prob_arrays[1].astype(np.float32)
    mk1 = (lambda: mrc_obj(objA)) if maps is None else maps[0]
    mk2 = (lambda: mrc_obj(objB)) if maps is None else maps[1]
    mrc1, mrc2 = mk1(), mk2()
    p1 = [mk1() for _ in range(4)]
    p2 = [mk2() for _ in range(4)]
    for k in range(4):
        p2[k].data = np.swapaxes(prob_maps_chain[:, :, :, k], 0, 2)
        p1[k].data = np.swapaxes(prob_maps[:, :, :, k], 0, 2)
    print("\n###Generating Params for Resampling Density Map 1###")
    mrc1, mrc_N1 = mrc_set_vox_size(mrc1, threshold1, voxel_spacing)
    print("\n###Generating Params for Resampling Density Map 2###")
    mrc2, mrc_N2 = mrc_set_vox_size(mrc2, threshold2, voxel_spacing)
    print("\n###Generating Params for Resampling Probability Map 1###")
    n1p = [mrc_set_vox_size(p, th=0.0, voxel_size=voxel_spacing)[1] for p in p1]
    print("\n###Generating Params for Resampling Probability Map 2###")
    n2p = [mrc_set_vox_size(p, th=0.0, voxel_size=voxel_spacing)[1] for p in p2]
    mrc_list = [mrc_N1, mrc_N2] + n1p + n2p
    max_dim = np.max([m.xdim for m in mrc_list])
    for m in mrc_list:
        if m.xdim != max_dim:
            m.xdim = m.ydim = m.zdim = max_dim
            m.orig = m.cent - 0.5 * voxel_spacing * m.xdim
    for m in mrc_list:
        m.dens = np.zeros((max_dim ** 3, 1), dtype="float32")
        m.data = np.zeros((max_dim, max_dim, max_dim), dtype="float32")
        m.vec = np.zeros((max_dim, max_dim, max_dim, 3), dtype="float32")
    print("\n###Processing MAP1 Resampling###")
    mrc_N1 = fastVEC(mrc1, mrc_N1, dreso=bandwidth)
    n1p = [fastVEC(p, q, dreso=bandwidth) for p, q in zip(p1, n1p)]
    print("\n###Processing MAP2 Resampling###")
    mrc_N2 = fastVEC(mrc2, mrc_N2, dreso=bandwidth)
    n2p = [fastVEC(p, q, dreso=bandwidth) for p, q in zip(p2, n2p)]
    return search_map_fft_prob(n1p[0], n1p[1], n1p[2], n1p[3], mrc_N1, mrc_N2, n2p[0], n2p[1], n2p[2], n2p[3],
                               ang=angle_spacing, alpha=alpha, TopN=topN, num_proc=num_processors, vave=vave,
                               vstd=vstd, pave=pave, pstd=pstd, showPDB=showPDB, folder=folder)


def main(argv=None):
    args = build_parser().parse_args(argv)
    if args.command == "orig":
        threshold1 = 0.00 if args.t is None else args.t
        threshold2 = 0.00 if args.T is None else args.T
        print(args.a, args.b, threshold1, threshold2, args.g, args.s, args.A, args.N, args.S, args.M, args.E)
        return run_orig(mrc_obj(args.a), mrc_obj(args.b), threshold1, threshold2, args.g, args.s, args.A, args.N,
                        args.S, args.M, args.E, args.o)
    if args.command == "prob":
        threshold1 = 0.00 if args.t is None else args.t
        threshold2 = 0.00 if args.T is None else args.T
        vave = -10 if args.vav is None else args.vav
        vstd = -10 if args.vstd is None else args.vstd
        pave = -10 if args.pav is None else args.pav
        pstd = -10 if args.pstd is None else args.pstd
        print(args.a, args.b, args.a, args.b, threshold1, threshold2, args.g, args.s, args.A, args.N, args.S, args.M,
              args.E, args.alpha, vave, vstd, pave, pstd)
        if args.alpha == 0.0:
            return alpha_is_zero(args.a, args.b, threshold1, threshold2, args.g, args.s, args.A, args.N, args.S,
                                 args.M, args.E, args.o)
        return run_prob(args.a, args.b, args.npa, args.npb, threshold1, threshold2, args.g, args.s, args.A, args.N,
                        args.S, args.alpha, vave, vstd, pave, pstd, args.P, args.o)
    return None


if __name__ == "__main__":
    main()
