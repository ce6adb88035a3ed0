/*
 * gbrmsd — C ABI of the GB300 (sm_103a) RMSD library behind mdtraj_gb300.
 *
 * Every pointer argument named x, ref, out_*, g_* or *_ws is a DEVICE pointer
 * owned by the caller; the library allocates nothing on the device (scratch
 * is passed in as a workspace sized by the *_workspace_bytes queries).
 * `stream` is a cudaStream_t (NULL = legacy default stream).  All entry points
 * are asynchronous with respect to the host unless stated otherwise, return
 * GBRMSD_OK (0) on success and a negative GBRMSD_E_* code on failure, with a
 * message available from gbrmsd_last_error() (thread-local).
 *
 * Threads: the compute entry points may be called from several host threads
 * at once (mdtraj runs its kernels with the GIL released), each call with its
 * own workspace and normally its own stream; the library keeps no per-call
 * state anywhere else.  gbrmsd_stream_config_select and the gbrmsd_profile_*
 * calls change process-wide settings and must not race with other calls.
 *
 * Coordinates are float32 nanometres in one of two padded layouts:
 *   GBRMSD_ATOM_MAJOR  frame f, atom k, axis c at x[f*frame_stride + 3*k + c]
 *   GBRMSD_AXIS_MAJOR  frame f, axis c, atom k at x[f*frame_stride + c*n_padded + k]
 * with n_padded >= n_atoms, n_padded % 4 == 0, frame_stride % 4 == 0 and the
 * base pointer 16-byte aligned (the bulk-copy engine moves 16-byte units).
 * Padding atoms are ignored.  These mirror the reference's (n_real_atoms,
 * n_padded_atoms, rowstride) conventions of mdtraj/rmsd/include/theobald_rmsd.h:13-18.
 */
#ifndef GBRMSD_H_
#define GBRMSD_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBRMSD_OK 0
#define GBRMSD_E_INVALID -1     /* bad argument (shape, alignment, mode) */
#define GBRMSD_E_WORKSPACE -2   /* workspace missing or too small */
#define GBRMSD_E_CUDA -3        /* CUDA runtime error (launch, copy) */
#define GBRMSD_E_DEVICE -4      /* a kernel reported a device-side error */
#define GBRMSD_E_UNSUPPORTED -5 /* device is not sm_103 / feature missing */

#define GBRMSD_ATOM_MAJOR 0
#define GBRMSD_AXIS_MAJOR 1

/* Streaming modes (what the per-frame pass computes). */
#define GBRMSD_MODE_CENTER 0      /* md.rmsd default: centre + trace + QCP      */
#define GBRMSD_MODE_PRECENTERED 1 /* frames centred, traces supplied: QCP only  */
#define GBRMSD_MODE_NOSUPERPOSE 2 /* md.rmsd(superpose=False)                   */

/* Library identification. */
int gbrmsd_version(void);
const char* gbrmsd_last_error(void);

/* 1 if the current device can run this library (sm_103), else 0. */
int gbrmsd_device_supported(void);

/* Device attributes of the current device, in this order: cc major, cc minor,
 * SMs, max opt-in shared memory per block, pageable memory access, pageable
 * access uses host page tables, concurrent managed access, host register
 * supported, direct managed access from host, L2 bytes, SM clock kHz, memory
 * clock kHz.  Writes min(n, count) values (-1 when unknown), returns count. */
int gbrmsd_device_caps(int32_t* caps, int32_t n);

/* ---- Reference preparation ------------------------------------------------
 * Replaces inplace_center_and_trace_atom_major(ref, &g, 1, n)
 * (mdtraj/rmsd/include/center.h:7-8, called at mdtraj/rmsd/_rmsd.pyx:213) for
 * the reference frame, and additionally lays the reference out for the
 * streaming kernels.  ref_xyz: raw (n_atoms, 3) atom-major frame on device.
 * centre = 1: subtract the float centroid (double mean rounded to float, as the
 * reference does); centre = 0: copy as is (precentered / no-superpose use).
 */
size_t gbrmsd_reference_workspace_bytes(int32_t n_atoms, int32_t n_padded);
int gbrmsd_prepare_reference(const float* ref_xyz, int32_t n_atoms, int32_t n_padded,
                             int32_t layout, int32_t centre, void* ref_ws, size_t ref_ws_bytes,
                             void* stream);
/* Copies the prepared reference's float trace and centroid to host memory
 * (synchronises `stream`).  Either output may be NULL. */
int gbrmsd_reference_info(const void* ref_ws, float* host_trace, float* host_centroid3,
                          void* stream);

/* ---- RMSD of every frame to one reference ---------------------------------
 * mode GBRMSD_MODE_CENTER replaces the centre + prange(msd_atom_major) + sqrtf
 * loop of md.rmsd (mdtraj/rmsd/_rmsd.pyx:211-224): frames are NOT modified;
 * out_centroid (n_frames x 3 float, optional) receives the centroids the
 * reference would subtract in place, out_trace (optional) the traces.
 * mode GBRMSD_MODE_PRECENTERED replaces the prange loops over msd_axis_major
 * / msd_atom_major of getMultipleRMSDs_axis_major / _atom_major
 * (_rmsd.pyx:546-550, :606-609): g_target holds the per-frame traces and g_ref
 * the reference trace; self_index = the frame whose storage is the reference
 * (the reference's pointer-equality shortcut, theobald_rmsd_generic.h:22-23),
 * or -1.
 * mode GBRMSD_MODE_NOSUPERPOSE replaces msd_nosuperpose (_rmsd.pyx:762-793);
 * the reference must then be prepared with centre = 0.
 * ws: device workspace of at least gbrmsd_rmsd_workspace_bytes(...) bytes.
 */
size_t gbrmsd_rmsd_workspace_bytes(int64_t n_frames, int32_t n_atoms);
int gbrmsd_rmsd_to_reference(const float* x, int64_t n_frames, int32_t n_atoms, int32_t n_padded,
                             int64_t frame_stride, int32_t layout, int32_t mode,
                             const void* ref_ws, const float* g_target, float g_ref,
                             int64_t self_index, float* out_rmsd, float* out_centroid,
                             float* out_trace, void* ws, size_t ws_bytes, void* stream);

/* Allocation-free variant of gbrmsd_rmsd_to_reference.  It has no
 * counterpart in the reference (mdtraj's CPU path never allocates device
 * memory).  For callers that cannot allocate device memory at the point they
 * need RMSDs -- code inside another runtime's memory pool (the pool owns the
 * device memory), a plugin whose host application hands it buffers but no
 * allocator, or a loop that must not call cudaMalloc/cudaFree (they can
 * synchronise the whole device) -- the scratch is a
 * fixed 16 MiB device array inside the library (held by every GPU that loads
 * the library until the process exits), so the call takes no workspace and
 * calls no allocator.  Limit: gbrmsd_noalloc_max_frames(n_atoms) frames per
 * call (about 68,700 on a 152-SM GB300, for any atom count); larger requests
 * fail with GBRMSD_E_WORKSPACE before any work is queued.  The first call on a
 * device resolves the array's address with that device current and should
 * come before any stream capture; the address is kept for the life of the
 * process, so the entry point must not be used after a cudaDeviceReset.
 * Calls share the array: work of two calls that overlaps on the GPU races, so
 * serialise them.  Arguments as for gbrmsd_rmsd_to_reference. */
int gbrmsd_rmsd_to_reference_noalloc(const float* x, int64_t n_frames, int32_t n_atoms, int32_t n_padded,
                                     int64_t frame_stride, int32_t layout, int32_t mode,
                                     const void* ref_ws, const float* g_target, float g_ref,
                                     int64_t self_index, float* out_rmsd, float* out_centroid,
                                     float* out_trace, void* stream);

/* Error word of the last gbrmsd_rmsd_to_reference_noalloc on the current
 * device (it lives in the library's static scratch, which such callers cannot
 * reach through a workspace pointer): synchronises `stream`, writes the word
 * to *word when word is not NULL (bit 1 = a bounded wait expired, bit 2 =
 * non-finite input) and returns GBRMSD_E_DEVICE when it is non-zero.  No
 * reference counterpart.  gbrmsd_noalloc_max_frames: the largest frame count
 * one call accepts for frames of n_atoms atoms on the current device. */
int gbrmsd_noalloc_status(int32_t* word, void* stream);
int64_t gbrmsd_noalloc_max_frames(int32_t n_atoms);

/* ---- All-pairs RMSD matrix --------------------------------------------------
 * Replaces the clustering loop over md.rmsd(traj, traj, i, precentered=True)
 * (mdtraj examples/clustering.ipynb, cell 6; _rmsd.pyx:64-243 per row): out is
 * the symmetric n_frames x n_frames float32 matrix (row-major, diagonal 0).
 * centre = 1 centres every frame first (float centroid, as
 * Trajectory.center_coordinates); 0 uses the coordinates as given.
 * method 0: FP32 CUDA-core tiles; method 1: split-BF16 (hi + lo) tcgen05
 * tensor-core tiles with FP32 accumulation.  Both solve QCP per pair in FP32;
 * near-identical pairs (rmsd below 0.75 * scale / sqrt(n_atoms), scale = the
 * pair's mean squared distance of an atom from its centroid) are recomputed
 * exactly (compensated inner products, FP64 QCP, direct residual), any
 * number of them: pairs beyond the workspace's list of 2^22 are found again
 * by a scan of the output.  ws: gbrmsd_allpairs_workspace_bytes(...).
 */
size_t gbrmsd_allpairs_workspace_bytes(int64_t n_frames, int32_t n_atoms);
int gbrmsd_allpairs(const float* x, int64_t n_frames, int32_t n_atoms, int32_t n_padded, int64_t frame_stride,
                    int32_t layout, int32_t centre, int32_t method, float* out, void* ws, size_t ws_bytes,
                    void* stream);

/* Synchronises `stream`; reports how many pairs the last gbrmsd_allpairs (or
 * gbrmsd_cross_rmsd) on this workspace refined exactly (clamped to
 * INT32_MAX) and whether a device error was recorded. */
int gbrmsd_allpairs_status(const void* ws, int32_t* refined_pairs, void* stream);

/* ---- Superposition: rotations, in-place alignment, RMSF --------------------
 * gbrmsd_rotations: the optimal rotation of every frame's alignment atoms onto
 * a prepared reference -- the computeRot = 1 branch of msdFromMandG
 * (src/theobald_rmsd.cpp:279-332) as driven by superpose_atom_major,
 * rmsf and getMultipleAlignDisplaceRMSDs_atom_major (_rmsd.pyx:246-759).
 * out_rot[9 f ..] is R, row-major, with R (a - mu_f) the frame aligned onto
 * the reference (this equals the reference's own `rot` array for the
 * frame-vs-reference call order of getMultipleAlignDisplaceRMSDs_atom_major).
 * mode CENTER centres each frame on its own centroid (FP64, written to
 * out_centroid if given); PRECENTERED uses the coordinates as given with the
 * traces g_target / g_ref.  out_rmsd (optional) receives the RMSD as
 * gbrmsd_rmsd_to_reference would.  ws: gbrmsd_rotations_workspace_bytes.
 *
 * gbrmsd_apply_rotations: in place, every atom of every frame (atom-major,
 * frame_stride floats apart): x <- R_f (x - mu_f) + offset, where
 * (x - mu_f) and (y + offset) are rounded to float as from FP64 (within one
 * float ulp; Trajectory.superpose, core/trajectory.py:1127-1165, with
 * rot_atom_major, src/rotation_generic.h:29-44).  centroids (n_frames x 3
 * doubles, device) and offset3 (3 doubles, host) may be null (zero).  If
 * nonzero0 (device int) is given it is set to 1 when any rotated coordinate of
 * frame 0 is non-zero (the reference's overflow check,
 * core/trajectory.py:1157-1163).
 *
 * gbrmsd_rmsf: per-atom root-mean-square fluctuation over the frames of x
 * (atom-major), each frame first rotated about the origin by R_f when rot is
 * given (rmsf, _rmsd.pyx:419-451: mean position per atom, then mean squared
 * deviation).  ws: gbrmsd_rmsf_workspace_bytes.
 *
 * gbrmsd_rotated_rmsd: out[f] = sqrt(sum_k |R_f x_fk - ref_k|^2 / n_atoms)
 * (rot_msd_atom_major, src/rotation_generic.h:47-103, as used by
 * getMultipleAlignDisplaceRMSDs_atom_major); ref_frame is n_atoms x 3 floats.
 */
size_t gbrmsd_rotations_workspace_bytes(int64_t n_frames, int32_t n_atoms);
int gbrmsd_rotations(const float* x, int64_t n_frames, int32_t n_atoms, int32_t n_padded, int64_t frame_stride,
                     int32_t layout, int32_t mode, const void* ref_ws, const float* g_target, float g_ref,
                     float* out_rot, double* out_centroid, float* out_rmsd, void* ws, size_t ws_bytes,
                     void* stream);
int gbrmsd_apply_rotations(float* x, int64_t n_frames, int32_t n_atoms, int64_t frame_stride, const float* rot,
                           const double* centroids, const double* offset3, int32_t* nonzero0, void* stream);
size_t gbrmsd_rmsf_workspace_bytes(int64_t n_frames, int32_t n_atoms);
int gbrmsd_rmsf(const float* x, int64_t n_frames, int32_t n_atoms, int64_t frame_stride, const float* rot,
                float* out_rmsf, void* ws, size_t ws_bytes, void* stream);
int gbrmsd_rotated_rmsd(const float* x, int64_t n_frames, int32_t n_atoms, int64_t frame_stride, const float* rot,
                        const float* ref_frame, float* out_rmsd, void* stream);

/* ---- XTC trajectories decoded on the GPU -----------------------------------
 * Replaces the reference's XTC reader (formats/xtc/xtc.pyx over
 * xdrfile_xtc.c:38-87 and the coordinate decompression of xdrfile.c:779-998)
 * for feeding frames to the RMSD kernels without a host decode.
 * gbrmsd_xtc_index (host only): scans the XDR frame headers of `data`
 * (nbytes of an XTC file or of a chunk of one starting at a frame boundary),
 * writes up to `capacity` frame byte offsets, the number of complete frames,
 * their atom count (all frames must match) and the bytes they span
 * (`consumed`; a truncated last frame is left out).
 * gbrmsd_xtc_decode: one thread per frame decodes `data` (device copy) at the
 * given offsets (device) into xyz (device, atom-major, frame_stride floats per
 * frame), with optional step / time / box (9 floats) per frame and a status
 * per frame (0 ok; 1 bad magic, 2 atom count, 3 truncated or overrun, 4 bad
 * small-integer index).  Coordinates equal the reference reader's: integer
 * coordinate times float(1 / precision), in float. */
int gbrmsd_xtc_index(const uint8_t* data, int64_t nbytes, int64_t* offsets, int64_t capacity, int64_t* n_frames,
                     int32_t* n_atoms, int64_t* consumed);
int gbrmsd_xtc_decode(const uint8_t* data, int64_t nbytes, const int64_t* offsets, int64_t n_frames, int32_t n_atoms,
                      float* xyz, int64_t frame_stride, int32_t* step, float* time, float* box, int32_t* status,
                      void* stream);

/* ---- Cross RMSD: query frames against a resident database ------------------
 * Replaces `[md.rmsd(db[a:b], queries, k, precentered=True) for k in ...]`
 * (_rmsd.pyx:64-243 per query frame) for many requests at once.  A frame set
 * is a device buffer of prepared frames: centred float rows, split BF16 planes
 * and FP64 traces, laid out for `capacity` frames of n_atoms atoms, filled by
 * gbrmsd_frameset_prepare (rows [first, first + n_frames), any number of calls;
 * centre as in gbrmsd_allpairs).
 *
 * gbrmsd_cross_rmsd scores, for every request r, its n_query frames (rows
 * [pool0, pool0 + n_query) of the query set) against the database frames
 * [db0, db1):  out_r[q * (db1 - db0) + (i - db0)] = rmsd(db frame i, query
 * frame pool0 + q), float32, optimal superposition.  Requests may overlap in
 * the database and share tiles (their query rows must not overlap); each
 * result depends only on its own two frames.  method 0: FP32 CUDA-core tiles;
 * method 1: split-BF16 tcgen05 tiles.  Near-identical pairs are recomputed
 * exactly, as in gbrmsd_allpairs.  Errors and the refined-pair count are read
 * with gbrmsd_allpairs_status(ws, ...).  No counterpart in the reference: it
 * has no multi-reference call. */
typedef struct gbrmsd_cross_request {
  float* out;      /* device, n_query x (db1 - db0) float32 */
  int64_t pool0;   /* first query-set row */
  int64_t db0;     /* database frames [db0, db1) */
  int64_t db1;
  int32_t n_query;
  int32_t reserved;
} gbrmsd_cross_request_t;

size_t gbrmsd_frameset_bytes(int64_t capacity, int32_t n_atoms);
int gbrmsd_frameset_prepare(const float* x, int64_t n_frames, int32_t n_atoms, int32_t n_padded,
                            int64_t frame_stride, int32_t layout, int32_t centre, void* set, int64_t capacity,
                            int64_t first, void* stream);
size_t gbrmsd_cross_workspace_bytes(int64_t n_db, int64_t query_capacity, int32_t n_requests);
int gbrmsd_cross_rmsd(const void* db_set, int64_t db_capacity, int64_t n_db, const void* query_set,
                      int64_t query_capacity, int32_t n_atoms, const gbrmsd_cross_request_t* requests,
                      int32_t n_requests, int32_t method, void* ws, size_t ws_bytes, void* stream);

/* ---- Ragged batch: many trajectories in one launch -------------------------
 * Each segment s is a trajectory of seg_frames[s] frames of seg_atoms[s] atoms
 * (padded to seg_padded[s], a multiple of 4), atom-major, starting at float
 * offset seg_x_offsets[s] (multiple of 4) of one packed device buffer, scored
 * against its own frame 0 -- the work of `[md.rmsd(t, t, 0) for t in trajs]`
 * (_rmsd.pyx:211-224 per trajectory).  Output: one float per frame, segments
 * concatenated in order.
 *   gbrmsd_ragged_plan   host only: validates the segments, picks the launch
 *                        configuration (config in [0, gbrmsd_ragged_config_count()),
 *                        max_unit_quads = largest work unit in 4-atom quads;
 *                        <= 0 picks defaults) and sizes the workspace;
 *   gbrmsd_ragged_setup  uploads the segment tables and prepares every
 *                        segment's reference (synchronises `stream`);
 *   gbrmsd_ragged_rmsd   one persistent launch + QCP finish + refinement;
 *                        kernels and a memset only, so it can be captured in
 *                        a CUDA graph and replayed.
 */
typedef struct gbrmsd_ragged_plan {
  int32_t n_seg;
  int32_t config;
  int32_t max_unit_quads;
  int32_t grid;
  int64_t total_frames;
  int64_t total_units;
  size_t ws_bytes;
} gbrmsd_ragged_plan_t;

int gbrmsd_ragged_config_count(void);
int gbrmsd_ragged_plan(const int64_t* seg_x_offsets, const int32_t* seg_atoms, const int32_t* seg_padded,
                       const int64_t* seg_frames, int32_t n_seg, int32_t config, int32_t max_unit_quads,
                       gbrmsd_ragged_plan_t* plan);
int gbrmsd_ragged_setup(const float* x, const int64_t* seg_x_offsets, const int32_t* seg_atoms,
                        const int32_t* seg_padded, const int64_t* seg_frames, const gbrmsd_ragged_plan_t* plan,
                        void* ws, size_t ws_bytes, void* stream);
int gbrmsd_ragged_rmsd(const float* x, float* out, const gbrmsd_ragged_plan_t* plan, void* ws, size_t ws_bytes,
                       void* stream);

/* ---- In-place centring ------------------------------------------------------
 * Replaces inplace_center_and_trace_atom_major (mdtraj/rmsd/include/center.h:7-8;
 * src/center_generic.h:3-44) for whole trajectories on the device, i.e. the
 * work of _center_inplace_atom_major (_rmsd.pyx:487-491) and
 * Trajectory.center_coordinates (mdtraj/core/trajectory.py:2114-2137):
 * centroid = double mean rounded to float, x -= centroid in float, trace =
 * sum of float squares accumulated in extended precision, stored as float.
 */
int gbrmsd_center_inplace(float* x, int64_t n_frames, int32_t n_atoms, int32_t n_padded,
                          int64_t frame_stride, int32_t layout, float* out_traces,
                          float* out_centroids, void* ws, size_t ws_bytes, void* stream);

/* Mass-weighted centring: replaces the mass_weighted=True branch of
 * Trajectory.center_coordinates (mdtraj/core/trajectory.py:2133-2134, with
 * compute_center_of_mass, mdtraj/geometry/distance.py:366-384).  x is
 * atom-major (frame_stride floats apart, no padding needed); weights are the
 * n_atoms normalised masses (doubles, device, summing to 1 as the reference
 * normalises them).  Per frame com = sum_k w_k x_k (to ~2^-48 relative) and
 * x <- float(x - com) in place; out_com (n_frames x 3 doubles, device) may be
 * null.  No workspace; traces are not computed (the reference's assignment
 * to xyz drops them). */
int gbrmsd_center_weighted_inplace(float* x, int64_t n_frames, int32_t n_atoms, int64_t frame_stride,
                                   const double* weights, double* out_com, void* stream);

/* Synchronises `stream` and returns GBRMSD_E_DEVICE if a kernel that used
 * this workspace recorded a device-side error (e.g. a bounded wait expired),
 * GBRMSD_OK otherwise.  The error word is cleared by the next call.
 * gbrmsd_workspace_error_word writes the word itself: bit 1 (value 1) = a
 * bounded wait expired (the results of that call are not valid); bit 2
 * (value 2) = some frame had non-finite coordinates (its RMSD is 0, as the
 * reference's clamp of a NaN msd gives, src/theobald_rmsd.cpp:275-277). */
int gbrmsd_workspace_status(const void* ws, void* stream);
int gbrmsd_workspace_error_word(const void* ws, int32_t* word, void* stream);

/* ---- Failure detection ------------------------------------------------------
 * Every wait of the streaming kernels on a bulk copy is bounded in wall time
 * (the GPU's global timer); when a wait runs out the kernel records bit 1 in
 * the error word, waits (bounded) for its copies still in flight and returns,
 * so the context stays usable and the caller sees GBRMSD_E_DEVICE from the
 * status calls.  The reference has no counterpart (its CPU loops cannot
 * stall; its only failure report is a printed warning, theobald_rmsd.cpp:
 * 195-215).  Process-wide settings: do not change them while other calls run.
 *   gbrmsd_set_wait_limit_ns  limit of each bounded wait (0 = default 2 s;
 *                             1 us .. 60 s); read at each launch.
 *   gbrmsd_test_skip_copy     test hook: the streaming kernel of later
 *                             gbrmsd_rmsd_to_reference calls never issues the
 *                             first copy of work unit `unit` (-1 = off), so a
 *                             wait runs out with nothing in flight.  Accepted
 *                             only while the wait limit is <= 100 ms. */
int gbrmsd_set_wait_limit_ns(uint64_t ns);
int gbrmsd_test_skip_copy(int64_t unit);

/* Launch configurations of the streaming kernel (warps per CTA, quads per
 * stage, stages per warp, reference in shared memory, reserved = 0).  By default the first configuration whose shared
 * memory fits is used; select(i) forces configuration i for later calls
 * where it fits (-1 restores the default); used by the tuner.  describe()
 * writes the 5 parameters and returns 1 if the configuration fits frames of
 * n_atoms atoms, 0 if not. */
int gbrmsd_stream_config_count(void);
int gbrmsd_stream_config_select(int32_t index);
int gbrmsd_stream_config_describe(int32_t index, int32_t n_atoms, int32_t* out5);

/* Timing of the dominant kernel of gbrmsd_rmsd_to_reference (streaming
 * kernel) and gbrmsd_allpairs (tile kernel) with CUDA events recorded on the
 * caller's stream, for benchmarks.  gbrmsd_profile_enable(n) arms recording for the next n
 * calls (0 disables; n <= 4096); gbrmsd_profile_read waits for the recorded
 * calls, writes up to `capacity` kernel times in milliseconds, re-arms, and
 * returns how many it wrote (negative on error).  Not thread-safe. */
int gbrmsd_profile_enable(int32_t max_calls);
int gbrmsd_profile_read(float* stream_kernel_ms, int32_t capacity);

/* ---- Host<->device plumbing used by the drop-in ---------------------------
 * Strided copy of n_rows rows of row_bytes bytes (cudaMemcpy2DAsync); kind:
 * 1 = host->device, 2 = device->host, 3 = device->device. */
int gbrmsd_copy_rows(void* dst, size_t dst_pitch, const void* src, size_t src_pitch,
                     size_t row_bytes, size_t n_rows, int32_t kind, void* stream);

/* 1 when kernels on the current device can read and write pageable host
 * memory through the host page tables (Grace + NVLink-C2C), else 0. */
int gbrmsd_pageable_access(void);

/* Page-locks [p, p + bytes) of caller-owned host memory for the device
 * (cudaHostRegister) / releases it (cudaHostUnregister, p as registered).
 * The streaming drop-in locks a large host array range by range, ahead of the
 * kernels that read and write it: on GB300 the GPU then reaches those pages
 * through its own page tables instead of translating every access through
 * the host's (measured on a 24 GB array after other processes had streamed
 * pageable memory: 186-200 ms per md.rmsd locked, 400-1,000 ms unlocked).
 * Returns GBRMSD_E_UNSUPPORTED (and touches nothing) when the range cannot be
 * locked, e.g. because the caller has locked it already. */
int gbrmsd_host_register(void* p, size_t bytes);
int gbrmsd_host_unregister(void* p);

/* Kernel-based strided row copy: dst row r (dst_pitch floats apart) gets
 * src row r (src_pitch floats apart, row_floats values), then zeros up to
 * dst_fill floats.  Either side may be pageable host memory when
 * gbrmsd_pageable_access() is 1 (unregistered host pointers are refused
 * otherwise).  Used by the drop-in to move numpy coordinates into the
 * padded device layout without a staged pageable memcpy. */
int gbrmsd_copy_rows_kernel(float* dst, int64_t dst_pitch, const float* src, int64_t src_pitch, int64_t row_floats,
                            int64_t dst_fill, int64_t n_rows, void* stream);

/* The reference's in-place centring side effect (src/center_generic.h:33-38,
 * x -= (float)centroid in float) written by a kernel straight into the
 * caller's HOST array (n_frames x n_atoms x 3, unpadded) from the device copy
 * of the same coordinates (atom-major, dev_frame_stride floats apart) and the
 * centroids of gbrmsd_rmsd_to_reference.  Needs gbrmsd_pageable_access()
 * for pageable host memory. */
int gbrmsd_write_centred(float* host, const float* dev, int64_t dev_frame_stride, const float* centroids,
                         int64_t n_frames, int32_t n_atoms, void* stream);

/* Host-side replica of the reference's in-place centring side effect
 * (src/center_generic.h:33-38: x -= (float)centroid, in float) on a HOST
 * atom-major array, using centroids produced by gbrmsd_rmsd_to_reference.
 * Multithreaded (n_threads <= 0: all hardware threads); synchronous. */
int gbrmsd_host_subtract_centroids(float* x, int64_t n_frames, int32_t n_atoms, int64_t frame_stride,
                                   const float* centroids, int32_t n_threads);

#ifdef __cplusplus
}
#endif

#endif /* GBRMSD_H_ */
