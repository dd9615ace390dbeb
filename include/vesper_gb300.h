/*
 * vesper_gb300.h -- C ABI of the GB300 (sm_103a) VESPER alignment hot path.
 *
 * Plain pointers and sizes only.  Unless stated otherwise every array
 * argument is DEVICE memory owned by the caller, laid out C-order with the
 * reference's [x][y][z] voxel indexing (VESPER_1_prob_new.py:43), and every
 * call is asynchronous on ``stream`` (a cudaStream_t passed as void*; NULL
 * means the legacy default stream).  No entry point allocates device memory:
 * scratch space is a caller-provided ``workspace`` whose size the matching
 * ``*_workspace_size`` call reports.  Every call returns a vesper_status;
 * vesper_last_error() gives a one-line message for the calling thread.
 *
 * The reference is a Python program with no FFI; each entry point below
 * replaces the reference function cited beside it, with the same argument
 * meaning, and the Python host layer (vesper_python_gb300/vesper.py) keeps
 * the reference's function names and raises where the reference raises.
 */
#ifndef VESPER_GB300_H
#define VESPER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum vesper_status {
    VESPER_OK = 0,
    VESPER_ERR_INVALID = 1,      /* bad argument (null pointer, size, mode)          */
    VESPER_ERR_UNSUPPORTED = 2,  /* grid side not supported by the kernels           */
    VESPER_ERR_CUDA = 3,         /* CUDA launch/runtime error                        */
    VESPER_ERR_WORKSPACE = 4,    /* workspace too small                              */
    VESPER_ERR_DEVICE = 5        /* a kernel reported an error through its status word */
};

/* Search modes (main.py:194-203 letters V/O/C/P/L, plus the prob search). */
enum vesper_mode {
    VESPER_MODE_VEC = 0,        /* 'V' VecProduct: 3 vector channels               */
    VESPER_MODE_OVERLAP = 1,    /* 'O' Overlap                                      */
    VESPER_MODE_CC = 2,         /* 'C' CC                                           */
    VESPER_MODE_PCC = 3,        /* 'P' PCC                                          */
    VESPER_MODE_LAPLACIAN = 4,  /* 'L' Laplacian                                    */
    VESPER_MODE_PROB = 5        /* prob search: 3 vector + 4 probability channels   */
};

/* Library version (major*10000 + minor*100 + patch). */
int vesper_version(void);

/* Message of the last failing call on this thread ("" if none). */
const char *vesper_last_error(void);

/* Largest grid side ``dim`` the search kernels accept for ``mode``. */
int vesper_max_dim(int mode);

/* Measurement helper (no counterpart in the reference): launches
 * blocks x threads threads that each run independent float32 FMA chains for
 * ``iters`` steps on ``stream``; *flops_out (HOST) receives the launch's
 * floating-point operations, so events around the call give the device's
 * FP32 FMA rate.  ``out`` is DEVICE float[blocks] (written only in a case no
 * input reaches). */
int vesper_fp32_peak_probe(int blocks, int threads, int iters, float *out, double *flops_out, void *stream);

/* FFT length rule of the grid side: 1 if ``n`` = 2^a 3^b 5^c 7^d 11^e 13^f
 * with e+f <= 1 (pyFFTW next_fast_len, VESPER_1_prob_new.py:97), else 0. */
int vesper_fast_len_ok(int n);

/* ---------------------------------------------------------------------------
 * Map preparation: the threshold and radius of mrc_set_vox_size
 * (VESPER_1_prob_new.py:72-89).  In place, data[data < th] = 0 (float32
 * compare; th < 0 acts as 0 and does not shift the data).  out2 is DEVICE
 * uint64[2]: out2[0] = the bits of the largest squared distance
 * ((i-cx)^2 + (j-cy)^2) + (k-cz)^2 (float64) of a non-zero voxel from the HOST
 * centre cent[3] (voxel units, [x][y][z] indexing); out2[1] = the number of
 * non-zero voxels (0: the reference's max() of an empty list raises).
 * ------------------------------------------------------------------------- */
int vesper_prepare_map(float *data, int sx, int sy, int sz, double threshold, const double *cent, uint64_t *out2,
                       void *stream);
/* vesper_prepare_map for nmap maps in one launch (per 64 maps): HOST arrays
 * data[nmap] (device pointers), dims[3 nmap], thresholds[nmap], cents[3 nmap];
 * out is DEVICE uint64[2 nmap], map i's pair at out[2i] -- the same values as
 * nmap calls of vesper_prepare_map. */
int vesper_prepare_maps(int nmap, float *const *data, const int *dims, const double *thresholds, const double *cents,
                        uint64_t *out, void *stream);

/* fastVEC statistics of a d^3 float64 density (VESPER_1_prob_new.py:157-161):
 * stats_out DEVICE double[5] = {sum, count != 0, mean of > 0, L2 norm of > 0,
 * L2 norm of (> 0 values - mean)}. */
int vesper_map_stats(const double *data, int dim, double *stats_out, void *stream);
/* The same statistics over many blocks, with a caller workspace of
 * vesper_map_stats_workspace_size bytes (chunk partial sums added in a fixed
 * order).  No counterpart in the reference. */
int vesper_map_stats_workspace_size(int dim, size_t *bytes);
int vesper_map_stats_ws(const double *data, int dim, double *stats_out, void *workspace, size_t workspace_bytes,
                        void *stream);

/* ---------------------------------------------------------------------------
 * fastVEC: Gaussian-weighted unit-vector field of one resampled map.
 * Replaces doFastVEC / calc (VESPER_1_prob_new.py:121-142, :180-257).
 *
 *   src        float32 [sx][sy][sz]   thresholded source density
 *   src_width  source voxel width (A)            src_orig  HOST double[3]
 *   dim        destination side d                dest_width coarse spacing s
 *   dest_orig  HOST double[3]                    dreso      bandwidth g
 *   data_out   double [d][d][d]   Gaussian-weighted density (0 where skipped)
 *   data_f32   float  [d][d][d]   optional float32 copy of data_out (NULL ok);
 *              prob mode stores the density as float32 (main.py:345)
 *   vec_out    float  [d][d][d][3] unit vectors (0 where skipped)
 * ------------------------------------------------------------------------- */
int vesper_fastvec_workspace_size(int sx, int sy, int sz, int dim, size_t *bytes);
int vesper_fastvec(const float *src, int sx, int sy, int sz, double src_width, const double *src_orig,
                   int dim, double dest_width, const double *dest_orig, double dreso,
                   double *data_out, float *data_f32, float *vec_out,
                   void *workspace, size_t workspace_bytes, void *stream);

/* ---------------------------------------------------------------------------
 * Rotation of the query map for ``nrot`` rotations.
 * Replaces rot_mrc (VESPER_1_prob_new.py:279-354) and, with ``probs``,
 * rot_mrc_prob (:1211-1299).
 *
 *   data     double [d][d][d]         vec  float [d][d][d][3]
 *   probs    float  [4][d][d][d] or NULL (each channel masked by its own != 0)
 *   rotmats  float  [nrot][3][3]  np.flip of the ZYX Euler matrix with
 *            |m| < 1e-15 zeroed, cast to float32 (VESPER_1_prob_new.py:305-310)
 *   data_out double [nrot][d][d][d], vec_out float [nrot][d][d][d][3],
 *   probs_out float [nrot][4][d][d][d] (only with probs)
 * ------------------------------------------------------------------------- */
int vesper_rot_gather(const double *data, const float *vec, const float *probs, int dim,
                      const float *rotmats, int nrot, double *data_out, float *vec_out, float *probs_out,
                      void *stream);

/* ---------------------------------------------------------------------------
 * Target spectra conj(rfftn(x_c)) of the target map's mode fields, computed
 * in float64 and stored as complex64 [C][d][d][d/2+1] (interleaved re, im).
 * Replaces the target set-up of search_map_fft (VESPER_1_prob_new.py:601-628)
 * and search_map_fft_prob (:846-864).  ``ave`` is the target's fastVEC
 * average (used by PCC).  For VESPER_MODE_PROB ``probs`` holds the four
 * target probability maps (float32 [4][d][d][d]).
 * ------------------------------------------------------------------------- */
int vesper_spectra_bytes(int dim, int mode, size_t *bytes);
int vesper_target_workspace_size(int dim, int mode, size_t *bytes);
int vesper_target_spectra(const double *data, const float *vec, const float *probs, int dim, int mode,
                          double ave, void *spectra_out, void *workspace, size_t workspace_bytes, void *stream);

/* ---------------------------------------------------------------------------
 * Rotational search: for every rotation r, rotate the query map, correlate it
 * with the target over all circular translations by FFT and keep the best
 * translation (largest score, first in C order).
 * Replaces the rotation loops of search_map_fft (VESPER_1_prob_new.py:644-655,
 * :724-736) over rot_and_search_fft (:1418-1459, fft_search_best_dot :464-491,
 * fft_search_score_trans_1d :529-565, laplacian_filter :494-526,
 * find_best_trans_list :357-374), and of search_map_fft_prob (:880-896,
 * :935-962, :1025-1080) over rot_and_search_fft_prob (:1462-1527,
 * find_best_trans_mixed :1530-1545).
 *
 *   spectra   output of vesper_target_spectra for the same dim and mode
 *   data, vec, probs   the query map (probs only for VESPER_MODE_PROB)
 *   ave       the TARGET's fastVEC average (PCC query transform, :1447-1450)
 *   rotmats   float [nrot][3][3] as for vesper_rot_gather
 *   mix       HOST double[5] {alpha, vstd, vave, pstd, pave} or NULL; only for
 *             VESPER_MODE_PROB, enabling the mixed z-score (pass 2)
 *   scores_out float [nrot][nscore] raw best scores (unnormalised correlation,
 *             before the 1/d^3 and CC/PCC scale factors the host applies)
 *   lin_out   int32 [nrot][nscore] linear index x*d*d + y*d + z of the best
 *             translation
 *   nscore = vesper_search_nscore(mode, mix != NULL): 1 for V/O/C/P/L;
 *            prob: {vec, prob} without mix, {vec, prob, mixed} with mix.
 *   batch     rotations resident per pipeline step (0 = library default)
 * ------------------------------------------------------------------------- */
int vesper_search_nscore(int mode, int with_mix);
int vesper_search_workspace_size(int dim, int mode, int batch, int nrot, size_t *bytes);
int vesper_search(const void *spectra, const double *data, const float *vec, const float *probs, int dim,
                  int mode, double ave, const float *rotmats, int nrot, const double *mix,
                  float *scores_out, int32_t *lin_out, int batch, void *workspace, size_t workspace_bytes,
                  void *stream);

/* vesper_search with explicit kernel choices, for the autotuner: HOST
 * opts[3] = {path (-1 automatic, 0 radix-stage passes, 1 register two-step
 * passes where compiled for this side and mode, 2 the fused single-kernel
 * search where compiled, 3 pass B (x-axis DFTs, product, group sums) as
 * split-BF16 tensor-core contractions with passes A and C as path 1, else 0;
 * sides 32 and 64), channels per pass-A block (0 automatic), columns per
 * pass-B block (0 automatic)}.  Automatic picks 2, else 1, else 0.  Paths
 * 0-2 give the same results up to float32 rounding of the FFT; path 3 carries
 * the split-BF16 error (about 1e-5 of a transform's magnitude).  After a path-3
 * call, vesper_search_status reports whether a tensor-core wait timed out. */
int vesper_search_tuned(const void *spectra, const double *data, const float *vec, const float *probs, int dim,
                        int mode, double ave, const float *rotmats, int nrot, const double *mix, float *scores_out,
                        int32_t *lin_out, int batch, void *workspace, size_t workspace_bytes, void *stream,
                        const int *opts);

/* Profiling form of vesper_search, for benchmarks: the same work, plus CUDA
 * events around every launch.  pass_ms HOST float[4] receives the summed
 * device time of the rotate+z+y passes, the x/correlation passes, the
 * inverse y+z/argmax passes and the final decode; pass_launches HOST int[4]
 * the number of launches of each.  Waits on events up to 16 batches behind
 * the launch front and at the end, so it returns with the stream drained.
 * Not re-entrant: one profiling call at a time per process.  opts as for
 * vesper_search_tuned (NULL: automatic). */
int vesper_search_profile(const void *spectra, const double *data, const float *vec, const float *probs, int dim,
                          int mode, double ave, const float *rotmats, int nrot, const double *mix,
                          float *scores_out, int32_t *lin_out, int batch, void *workspace, size_t workspace_bytes,
                          void *stream, float *pass_ms, int *pass_launches, const int *opts);

/* Status word of the last search that used this workspace (HOST *status_out:
 * 0 ok, 1 a tensor-core pass timed out and its results are not valid).
 * Synchronises the stream.  No counterpart in the reference. */
int vesper_search_status(const void *workspace, size_t workspace_bytes, int *status_out, void *stream);

/* Which kernel family vesper_search_tuned(opts) runs for this side and mode
 * (*path_out: 0 radix-stage, 1 register two-step, 2 fused, 3 tensor-core
 * pass B) and how many
 * kernel launches it makes for nrot rotations at this batch (0: default).
 * No counterpart in the reference. */
int vesper_search_plan(int dim, int mode, int batch, int nrot, const int *opts, int *path_out, int *launches_out);

/* vesper_search without a workspace argument.  No counterpart in the
 * reference: it serves callers that cannot allocate device memory
 * themselves (for example code running while a global-mode stream capture is
 * active elsewhere in the process, or a host application that provides only
 * pre-allocated inputs and outputs under a fixed device-memory budget).  Its
 * scratch is a fixed 16 MiB array inside this library, reserved on every GPU
 * that loads the library until the process exits; it allocates nothing.
 * Same arguments and results as vesper_search, run with the largest
 * pipeline batch whose scratch fits the array.  Rejects, with
 * VESPER_ERR_UNSUPPORTED, any call whose
 * vesper_search_workspace_size(dim, mode, 1, nrot) exceeds 16 MiB (mode V
 * fits up to dim 75 with the 24,624 rotations of a 10-degree grid).  The
 * first call on each device looks up the array's device address, and the
 * first call for each (mode, dim) loads that side's kernels and sets their
 * shared-memory limits: make one call for every (mode, dim) you will use
 * before any stream capture; after it, a call may itself be recorded into a
 * CUDA graph captured in global mode.  All calls share the array, so calls that
 * overlap on the GPU (other streams or host threads) race: serialise them. */
int vesper_search_static(const void *spectra, const double *data, const float *vec, const float *probs, int dim,
                         int mode, double ave, const float *rotmats, int nrot, const double *mix, float *scores_out,
                         int32_t *lin_out, void *stream);

/* ---------------------------------------------------------------------------
 * Stable top-N: indices of the ``topn`` largest of scores[i*stride]
 * (i < n), ties to the lower index -- Python's stable
 * sorted(..., reverse=True)[:N] (VESPER_1_prob_new.py:664, :739, :992, :1082).
 * idx_out int32 [topn]; entries past n are -1.
 * ------------------------------------------------------------------------- */
int vesper_topn(const float *scores, int n, int stride, int topn, int32_t *idx_out, void *stream);

/* ---------------------------------------------------------------------------
 * Final-model scoring in float64.  Replaces get_score
 * (VESPER_1_prob_new.py:1302-1393), including its ``d2 = where(d2 <= 0, 0,
 * d1)`` (:1357).
 *   tdata/tvec: target map; tave/tstd/tstd_norm_ave: its fastVEC statistics
 *   sdata/svec: rotated query map; trans: HOST int[3] best translation
 *   result_out double[8] = {Nm, total, cc/(std1*std2), pcc/(pstd1*pstd2),
 *                           DOT score, ave2, std2, pstd2}
 *   sco_out double [d][d][d] per-voxel dot products (NULL ok)
 * ------------------------------------------------------------------------- */
int vesper_rescore_workspace_size(int dim, size_t *bytes);
/* With a workspace of vesper_rescore_workspace_size bytes the sums run over
 * many blocks (chunk partials added in a fixed order); with workspace NULL
 * they run in one block and nothing but the outputs is written. */
int vesper_rescore(const double *tdata, const float *tvec, double tave, double tstd, double tstd_norm_ave,
                   const double *sdata, const float *svec, int dim, const int32_t *trans, double *result_out,
                   double *sco_out, void *workspace, size_t workspace_bytes, void *stream);
/* vesper_rescore for nmodel rotated query maps at once (no counterpart in the
 * reference: its loop calls get_score per model): sdata [nmodel][d^3],
 * svec [nmodel][d^3][3], trans_dev DEVICE int32 [nmodel][3] already wrapped
 * to (-d/2, d/2], result_out DEVICE double [nmodel][8].  Four launches for all
 * models. */
int vesper_rescore_batch_workspace_size(int dim, int nmodel, size_t *bytes);
int vesper_rescore_batch(const double *tdata, const float *tvec, double tave, double tstd, double tstd_norm_ave,
                         const double *sdata, const float *svec, int dim, const int32_t *trans_dev, int nmodel,
                         double *result_out, void *workspace, size_t workspace_bytes, void *stream);
/* vesper_rescore_batch with the target's statistics read from DEVICE memory
 * (tstats_dev: the double[5] that vesper_map_stats / vesper_map_stats_ws
 * write; ave, L2 norm and centred L2 norm are entries 2, 3 and 4), so that a
 * caller can record the call once and replay it for new maps without reading
 * the statistics back to the host.  No counterpart in the reference. */
int vesper_rescore_batch_dev(const double *tdata, const float *tvec, const double *tstats_dev, const double *sdata,
                             const float *svec, int dim, const int32_t *trans_dev, int nmodel, double *result_out,
                             void *workspace, size_t workspace_bytes, void *stream);

/* ---------------------------------------------------------------------------
 * Refinement on the device (the reference's refinement set and its top-N,
 * VESPER_1_prob_new.py:689-740, with get_score's wrapped translation,
 * :1323-1329), for callers that keep the whole alignment on the device.
 *
 * vesper_refine_slots: for n pairs with topn global top angles each, given as
 * grid indices tg int64 [n][topn] (-1: none) into grid_rows int64 [ngrid]
 * (each grid angle's row on a lattice of lattice_n steps per axis, row =
 * (x L + y) L + z, each in [0, L^3)), and offsets int64 [27][3] in lattice
 * steps, each in [-L, L) (the kernel reads lattice rows only within these
 * ranges; the reference's offsets are -1, 0 and +1): slot
 * t = (i topn + k) 27 + o is top k's row plus offset o, valid where
 * x < L, y < L, z < L/2 before negative coordinates wrap by +L and the top
 * exists.  Writes crow int64 [n topn 27] (0 for an invalid slot), valid uint8
 * [same] and rmats float [same][3][3] = lattice[crow] (lattice float
 * [L^3][3][3]).  All pointers DEVICE.
 *
 * vesper_refine_pick: one pair's slots after their search (scores float and
 * lin int32 [nslot][nscore], column 0 used): the stable top-N over the valid
 * slots (the others read -inf; ties to the lower slot; -1 past the slots) in
 * rtop int32 [topn], and per pick (slot 0 standing in for -1) its row int64,
 * score float, lin int64, rotation mats float [topn][3][3] = lattice[row] and
 * trans int32 [topn][3] = (lin / d^2, lin / d % d, lin % d), each t > d/2
 * taken as t - d.  All pointers DEVICE.  No counterparts in the reference.
 * ------------------------------------------------------------------------- */
int vesper_refine_slots(const int64_t *tg, int n, int topn, const int64_t *grid_rows, int ngrid, const int64_t *offsets,
                        int lattice_n, const float *lattice, int64_t *crow, uint8_t *valid, float *rmats,
                        void *stream);
int vesper_refine_pick(const float *scores, const int32_t *lin, int nscore, const uint8_t *valid, const int64_t *crow,
                       int nslot, int topn, const float *lattice, int d, int32_t *rtop, int64_t *rows, float *rscore,
                       int64_t *rlin, float *mats, int32_t *trans, void *stream);

/* ---------------------------------------------------------------------------
 * Probability-map hole filling (interpolate, interpolation_functions.py:6-135)
 * in place on a DEVICE float32 [nx][ny][nz][nch] array: the parity of the
 * first voxel (C order) with channel 0 > 0 fixes the sampled lattice; zero
 * voxels off it take the float64 mean of their neighbours along the axes
 * where their parity differs (one axis, then two, then three), rounded to
 * float32, with the reference's wrap of index -1 and its loop bounds.
 * workspace: DEVICE, >= 8 bytes.  vesper_prob_interpolate_found (after the
 * call, synchronising the stream) sets *found = 0 when no voxel had a
 * positive channel 0, in which case the data is unchanged (the reference
 * fails there on an unbound variable).
 * ------------------------------------------------------------------------- */
int vesper_prob_interpolate(float *data, int nx, int ny, int nz, int nch, void *workspace, size_t workspace_bytes,
                            void *stream);
int vesper_prob_interpolate_found(const void *workspace, int *found, void *stream);

/* ---------------------------------------------------------------------------
 * Learned rotation proposal (no counterpart in the reference): a 3-D
 * convolutional encoder over each map's fields and the rotational
 * correlation of the two feature fields at zero translation, which orders
 * the angle grid so that vesper_search correlates only its best fraction.
 * Activations are float32 [C][d][d][d]; W is bfloat16 [cout][cin][3][3][3]
 * (zero padding), accumulation in float32.
 * ------------------------------------------------------------------------- */
/* Network input of one map: out[4][dp][dp][dp] float32 (dp = ceil(d/pool)),
 * the channels vx, vy, vz and (data != 0) of a fastVEC result averaged over
 * pool^3 blocks (clipped at the grid edge). */
int vesper_prop_field(const double *data, const float *vec, int d, int pool, float *out, void *stream);
/* One layer over nmap maps stacked in memory: in [nmap][cin][d^3] ->
 * out [nmap][cout][d^3] (ReLU when relu != 0). */
int vesper_prop_conv_fwd(const float *in, int cin, const void *W, const float *bias, int cout, int d, int relu,
                         int nmap, float *out, void *stream);
/* Backward of one layer: din (NULL for the first layer) = input gradient;
 * dW, db ACCUMULATE (+=).  out is the layer's forward output (ReLU mask). */
int vesper_prop_conv_bwd(const float *dout, const float *out, int relu, const float *in, const void *W, int cin,
                         int cout, int d, float *din, float *dW, float *db, void *stream);
/* scores[r] = sum_k sum_v ET[k][v] * EQ[k][src_r(v)], src_r the reference's
 * nearest-voxel rotation gather (every in-bounds voxel accepted). */
int vesper_prop_score(const float *ET, const float *EQ, int K, int d, const float *rotmats, int nrot,
                      float *scores, void *stream);
/* Channel-major [nmap][K][d^3] -> voxel-major [nmap][d^3][K]. */
int vesper_prop_vmajor(const float *in, int K, int d, int nmap, float *out, void *stream);
/* vesper_prop_score on voxel-major features ([d^3][K], K a multiple of 4,
 * at most 32, 16-byte aligned): the inference form. */
int vesper_prop_score_vm(const float *ET, const float *EQ, int K, int d, const float *rotmats, int nrot,
                         float *scores, void *stream);
/* Inference form with float16 voxel-major features ([d^3][K] half, K a
 * multiple of 8, at most 32, 16-byte aligned), four rotations per block,
 * float32 accumulation; vesper_prop_vmajor_f16 writes that layout from
 * channel-major float32 [nmap][K][d^3]. */
int vesper_prop_vmajor_f16(const float *in, int K, int d, int nmap, void *out, void *stream);
int vesper_prop_score_f16(const void *ET, const void *EQ, int K, int d, const float *rotmats, int nrot,
                          float *scores, void *stream);
/* The gather geometry of every (rotation, voxel) of a d^3 grid, d^3 <= 32767:
 * srcmap_out int16 [nrot][d^3] (-1: none), computed once per grid and
 * rotation set; vesper_prop_score_map scores from it (float16 voxel-major
 * features as for vesper_prop_score_f16) without recomputing the geometry. */
int vesper_prop_srcmap(int d, const float *rotmats, int nrot, void *srcmap_out, void *stream);
int vesper_prop_score_map(const void *ET, const void *EQ, int K, int d, const void *srcmap, int nrot,
                          float *scores, void *stream);
/* vesper_prop_score_map for npair pairs of one grid side in one launch: VM is
 * float16 voxel-major [2 npair][d^3][K] (pair i: target map 2i, query map
 * 2i + 1), scores float32 [npair][nrot]; the same scores as npair calls of
 * vesper_prop_score_map, bit for bit. */
int vesper_prop_score_map_many(const void *VM, int npair, int K, int d, const void *srcmap, int nrot,
                               float *scores, void *stream);
int vesper_prop_score_bwd_workspace(int K, int d, size_t *bytes);
/* Gradients of sum_r gscores[r] * scores[r]; gET, gEQ ACCUMULATE (+=). */
int vesper_prop_score_bwd(const float *ET, const float *EQ, int K, int d, const float *rotmats, int nrot,
                          const float *gscores, float *gET, float *gEQ, void *workspace, size_t workspace_bytes,
                          void *stream);
/* u = scores standardised over the n rotations (mean 0, population std 1),
 * p = softmax(u / tau): loss += -sum target log p (DEVICE float[1]);
 * gscores = dloss/dscores through the standardisation. */
int vesper_prop_softmax_ce(const float *scores, const float *target, int n, float tau, float *loss, float *gscores,
                           void *stream);
/* Adam step on float32 master weights (gradient scaled by gscale), refreshing
 * the bfloat16 copy wbf16 when non-NULL. */
int vesper_prop_adam(float *w, float *m, float *v, const float *g, int n, float lr, float b1, float b2, float eps,
                     int step, float gscale, void *wbf16, void *stream);
/* idx_out int32[k]: indices of the k largest scores (ties to the lower
 * index), in ascending index order. */
int vesper_topk_subset(const float *scores, int n, int k, int32_t *idx_out, void *stream);
/* The same for nbatch score rows at once: scores float[nbatch][n] ->
 * idx_out int32[nbatch][k], one block per row. */
int vesper_topk_subset_batch(const float *scores, int nbatch, int n, int k, int32_t *idx_out, void *stream);

/* ---- split-BF16 tensor-core DFT (search pass B) -------------------------- */
/* Pass B of the search on the 5th-generation tensor cores, on caller-provided
 * spectra (device pointers, complex64):
 *   S [nbatch][nch][d][d][d/2+1]  x-untransformed spectra of the rotated query,
 *   T [nch][d][d][d/2+1]          conjugated target spectra,
 *   U [nbatch][ngrp][d][d][d/2+1] out: per score group g (channels [0, split)
 *                                 and [split, nch)) the inverse x DFT of
 *                                 sum_c T_c * DFT_x(S_c), unnormalised.
 * The x-axis DFTs run as split-BF16 contractions (hi*hi + hi*lo + lo*hi,
 * float32 accumulation).  d = 32 or 64.  *err (device int) is set to 1 if a
 * tensor-core wait timed out.  Replaces the float32 FFT pass B of the search
 * (fft_search_best_dot, VESPER_1_prob_new.py:464-491, and the prob-mode passes
 * :880-962) when the search option selects it. */
int vesper_tc_pass_b(const void *S, const void *T, void *U, int d, int nch, int ngrp, int split, int nbatch, int *err,
                     void *stream);
/* Failure self-test of the same kernel (one rotation): every CTA first waits
 * on a barrier that nothing completes, gives up after limit_ms (1..1000),
 * sets *err = 1, frees its TMEM and returns without touching U.  The context
 * stays usable.  No counterpart in the reference. */
int vesper_tc_pass_b_stall_test(const void *S, const void *T, void *U, int d, int nch, int ngrp, int split,
                                int limit_ms, int *err, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* VESPER_GB300_H */
