/* gapgpu.h -- C ABI of the GB300 GAP energy/force/virial library (libgapgpu.so).
 *
 * The library replaces the body of QUIP's IPModel_GAP_Calc
 * (src/Potentials/IPModel_GAP.f95:233-605) and the connection build it relies on
 * (connection_calc_connect, src/libAtoms/Connection.f95:1035-1310).  Everything above
 * it -- potential_calc (src/Potentials/Potential.f95:803-996), quippy's
 * Potential.calculate (quippy/quippy/potential.py:177-325), DynamicalSystem MD -- keeps
 * its signatures; a Fortran iso_c_binding module binds these symbols.
 *
 * Conventions (all match QUIP's Fortran arrays, so no copies are needed there):
 *   pos           double[3*n]   Fortran pos(3,N): pos[3*i + k]
 *   Z             int32[n]
 *   lattice       double[9]     Fortran lattice(3,3), COLUMNS are the cell vectors:
 *                               lattice[3*c + k] = component k of cell vector c
 *   pbc           int32[3]      at%is_periodic
 *   force         double[3*n]   Fortran f(3,N)
 *   virial        double[9]     Fortran virial(3,3), column-major
 *   local_virial  double[9*n]   Fortran local_virial(9,N) = reshape(virial_i, (/9/))
 * Any output pointer may be NULL (the Fortran `present()` test).
 *
 * Errors: every entry point returns 0 (GAPGPU_OK) or a positive error kind and never
 * aborts; gapgpu_last_error() gives the message of the calling thread's last failure
 * (the Fortran shim maps it to RAISE_ERROR, src/libAtoms/error.inc:61).
 *
 * Threading: one calculation at a time per context.  A model may be shared by several
 * contexts (one per CUDA stream) once created.  There is no CPU fallback: without a
 * usable sm_103a GPU every compute entry point returns GAPGPU_ERR_CUDA.
 */
#ifndef GAPGPU_H
#define GAPGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gapgpu_model gapgpu_model;
typedef struct gapgpu_context gapgpu_context;

enum gapgpu_status {
    GAPGPU_OK = 0,
    GAPGPU_ERR_ARG = 1,          /* bad argument (NULL handle, size mismatch, unknown args_str key) */
    GAPGPU_ERR_XML = 2,          /* GAP XML could not be read or is inconsistent */
    GAPGPU_ERR_UNSUPPORTED = 3,  /* model feature outside this library (descriptor type, covariance) */
    GAPGPU_ERR_CUDA = 4,         /* no usable GPU, or a CUDA call failed */
    GAPGPU_ERR_ATOMS = 5,        /* atoms rejected: negative cutoff, overlapping atoms, NaN positions */
    GAPGPU_ERR_TIMEOUT = 6       /* a bounded device-side wait gave up */
};

enum gapgpu_precision {
    GAPGPU_FP64 = 0,         /* plain path: every stage in FP64 */
    GAPGPU_MIXED_BF16X3 = 1, /* SOAP in FP32, kernel GEMMs as split-BF16 (hi*hi + hi*lo + lo*hi) on tcgen05 */
    GAPGPU_MIXED_TF32 = 2,   /* SOAP in FP32, both kernel GEMMs in TF32 on tcgen05 */
    GAPGPU_MIXED_F16 = 3     /* SOAP in FP32, both kernel GEMMs with FP16 operands on tcgen05 (10-bit mantissas
                                like TF32, at twice its rate) where the model allows it -- integer zeta, normalised
                                SOAP, bounded coefficients -- and in TF32 otherwise; the same context as
                                GAPGPU_MIXED_TF32 with the options gemm1_f16 = gemm2_f16 = 1 */
};

/* Message of the calling thread's last error ("" if none). */
const char* gapgpu_last_error(void);

/* Build a model from GAP XML text.  Replaces potential_Filename_Initialise
 * (src/Potentials/Potential.f95:438-468) + IPModel_GAP_Initialise_str
 * (src/Potentials/IPModel_GAP.f95:149-192): `label` selects the GAP_params stanza
 * (NULL/"" = first), sparseX_filename entries are resolved relative to `base_dir`
 * (the reference changes into the XML file's directory, Potential.f95:455-466).
 * `init_args` is the reference's init args_str (keys: label, E_scale, and
 * gap_variance_regularisation, which sets up the variance estimate of every coordinate as
 * IPModel_GAP.f95:170-187 does: K_MM + regularisation * I factorised once, in FP64). */
int gapgpu_model_create(const char* xml, size_t xml_len, const char* init_args, const char* base_dir,
                        gapgpu_model** out);

/* Potential cutoff = max descriptor cutoff (IPModel_GAP.f95:182-188). */
int gapgpu_model_cutoff(const gapgpu_model* model, double* cutoff);

/* Descriptor dimensions and sparse-point counts, for diagnostics and the autotuner. */
int gapgpu_model_info(const gapgpu_model* model, int* n_coordinates, int* dims, int* n_sparse, int capacity);

void gapgpu_model_destroy(gapgpu_model* model);

/* Per-stream evaluation context that owns the device workspace (neighbour lists,
 * descriptors, GEMM operands) and keeps it between calls. */
int gapgpu_context_create(const gapgpu_model* model, int precision, gapgpu_context** out);
int gapgpu_context_set_stream(gapgpu_context* ctx, void* cuda_stream);
void gapgpu_context_destroy(gapgpu_context* ctx);

/* The drop-in calculation: IPModel_GAP_Calc(this, at, e, local_e, f, virial,
 * local_virial, args_str) (IPModel_GAP.f95:233-241) with the connection built inside
 * (Potential.f95:844-858).  Host arrays in, host arrays out.  `atom_mask` (nullable)
 * is the logical property named by args_str atom_mask_name: it restricts the
 * centres (and the e0 sum) exactly as the reference does.  Recognised args keys:
 * atom_mask_name (value ignored here: pass the mask array), r_scale / E_scale
 * (rejected, as in IPModel_GAP.f95:348-350), xml_version, precision=fp64|bf16x3|tf32|fp16,
 * local_gap_variance=<name> / print_gap_variance=T (the variance estimate, read back with
 * gapgpu_gap_variance / gapgpu_gap_variance_instances; needs gap_variance_regularisation in
 * the model's init args).  Unknown keys are ignored, like
 * param_read_line(ignore_unknown=.true.). */
int gapgpu_calc(gapgpu_context* ctx, int n, const double* pos, const int32_t* Z, const double* lattice,
                const int32_t* pbc, const int32_t* atom_mask, double* energy, double* local_e, double* force,
                double* virial, double* local_virial, const char* args);

/* Same calculation with device-resident inputs and outputs on the context's stream
 * (no host synchronisation).  d_pos double[3n], d_Z int32[n]; lattice and pbc stay on
 * the host.  Outputs are device pointers (nullable).  Used by batching, serving and
 * device-resident MD, which keep positions in HBM between steps. */
int gapgpu_calc_device(gapgpu_context* ctx, int n, const double* d_pos, const int32_t* d_Z, const double* lattice,
                       const int32_t* pbc, double* d_energy, double* d_force, double* d_virial);

/* Batched evaluation of many independent structures in one pass (one neighbour build,
 * one SOAP/GEMM pipeline over every centre of the batch, per-structure reductions):
 * the loop over frames of quip / quippy's calculate over a list of Atoms
 * (quippy/quippy/potential.py:177-325) done as one GPU evaluation.  Structures are
 * concatenated: n_atoms[s] atoms each, pos double[3*sum n] and Z int32[sum n] in that
 * order, lattices double[9*nstruct] (columns are cell vectors), pbcs int32[3*nstruct].
 * Outputs (nullable): energies[nstruct], forces double[3*sum n], virials
 * double[9*nstruct].  Each structure's results are bit-identical to evaluating it alone
 * with the same context settings. */
int gapgpu_calc_batch(gapgpu_context* ctx, int nstruct, const int32_t* n_atoms, const double* pos, const int32_t* Z,
                      const double* lattices, const int32_t* pbcs, double* energies, double* forces, double* virials,
                      const char* args);

/* Context options: "graphs" (0/1): replay the evaluation phase from a CUDA graph when a
 * call has the same shapes and buffers as the previous one (captured on the second such
 * call); "timing" (0/1): per-stage CUDA events (gapgpu_context_timings); "priority"
 * (0/1): run on a stream of default or highest scheduling priority (latency-critical
 * requests next to background MD); "autotune" (0/1, default 1): time the tensor-core
 * GEMM's tile candidates on the first GEMM of each new shape and keep the fastest;
 * "pairs" (0/1/2, default 1, TF32 only): GEMM tiles on CTA pairs (256-row tiles computed
 * by two SMs, tcgen05 cta_group::2) -- 0 never, 1 as autotuner candidates next to the
 * single-CTA tiles (and the choice when no timing is possible), 2 only -- contexts whose
 * calls run at the same time as other contexts' (several streams) should set 0: CTA-pair
 * GEMMs issued from several streams at once stalled the device under load; "gemm2_f16" (0/1,
 * TF32 and FP16 contexts with pairs; default 1 for GAPGPU_MIXED_F16, 0 for
 * GAPGPU_MIXED_TF32): the second GEMM G = W X in FP16 (W' = S K^(zeta-1) and
 * X' = coef zeta / S x, both 10-bit mantissas in FP16's normal range) where the model
 * allows it (integer zeta, normalised SOAP, bounded S), else in TF32; "gemm1_f16" (0/1,
 * same defaults): the first GEMM K = Q X^T in FP16 as well (FP16 descriptors from the
 * forward kernel and FP16 sparse points, under the same conditions); "soap_fwd" (0/1,
 * default 1, FP32 SOAP): the forward with the basis size fixed at compile time where the
 * basis has an instance (l_max + 1 by n_max rounded up to 4: 9x12, 7x8, 5x8, 5x4), else
 * the generic forward; "soap_bwd" (0/1, default 1, FP32 SOAP): the backward as a
 * per-centre h kernel followed by one thread per neighbour pair where the basis has an
 * instance (the same sizes), else one block per centre.  Both choices give the same
 * results to FP32 rounding. */
int gapgpu_context_set_option(gapgpu_context* ctx, const char* key, int value);

/* energy_per_coordinate of the last gapgpu_calc / gapgpu_calc_batch whose args requested
 * it ("energy_per_coordinate=<name>", IPModel_GAP.f95:335): per structure and coordinate
 * (structure-major, model coordinate order) the sum of e_i * covariance_cutoff over the
 * evaluated descriptor instances, before E_scale and without e0 (:462, :570).  *count
 * receives nstruct * n_coordinates; GAPGPU_ERR_ARG when capacity is smaller or the last
 * evaluation did not request the sums.  The calc argument only_descriptor=<k> (:334,
 * :399-403) evaluates only coordinate k (1-based) of a model with more than one. */
int gapgpu_energy_per_coordinate(gapgpu_context* ctx, double* out, int capacity, int* count);

/* GAP variance estimate of the last gapgpu_calc whose args requested it
 * (local_gap_variance / print_gap_variance, IPModel_GAP.f95:330-335, :464-488):
 * local_variance[n] = sum over descriptor instances containing the atom of
 * sigma^2 fc^2 / |ci|, and variance_gradient[3n] (Fortran (3,N) layout) the property
 * gap_variance_gradient, the derivative of the summed local variances with respect to each
 * atom's position (available when that calculation computed forces or virials).
 * sigma^2 = k(x,x) - k^T (K_MM + lambda I)^-1 k is the sparse-GP predictive variance, in
 * FP64 whatever the context's precision.  Either output may be NULL. */
int gapgpu_gap_variance(gapgpu_context* ctx, double* local_variance, double* variance_gradient, int n);

/* The variance of every descriptor instance of coordinate `coordinate` (0-based) of that
 * calculation -- what print_gap_variance prints (IPModel_GAP.f95:506-516): sigma^2, the
 * squared covariance cutoff fc^2, and the instance's atoms (the centre and -1 for SOAP;
 * i and j of the directed pair i -> j for distance_2b).  Writes at most capacity entries
 * (NULL arrays skipped); *count receives the number of instances. */
int gapgpu_gap_variance_instances(gapgpu_context* ctx, int coordinate, double* variance, double* fc2, int32_t* atom_i,
                                  int32_t* atom_j, int capacity, int* count);

/* Text report of the autotuner's choices so far (one line per GEMM shape: chosen N tile
 * and the time of every candidate).  Returns the report length; writes at most
 * capacity-1 characters and a terminating NUL. */
int gapgpu_tuning_report(char* buf, int capacity);

/* Device memory one evaluation of n_atoms atoms with about mean_neighbours neighbours
 * each needs in a context of this precision (bytes, an estimate used for admission). */
int gapgpu_model_footprint(const gapgpu_model* model, int precision, int64_t n_atoms, double mean_neighbours,
                           int64_t* bytes);

/* Device-resident velocity-Verlet MD of nstruct independent replicas
 * (DynamicalSystem advance_verlet1/advance_verlet2, src/libAtoms/DynamicalSystem.f95:
 * 1814-2383, as run by DynamicalSystem_run, src/Potentials/Potential.f95:2304-2370),
 * with QUIP's skin rule for the connection (Connection.f95:1086-1125): lists are built
 * at cutoff + skin and refreshed (connection_calc_dists) until an atom has moved skin/2.
 * Layouts as gapgpu_calc_batch; velo in A/fs, mass per atom in eV fs^2/A^2 (amu times
 * MASSCONVERT), dt in fs.  The object owns its own context (gapgpu_md_context). */
typedef struct gapgpu_md gapgpu_md;
int gapgpu_md_create(const gapgpu_model* model, int precision, int nstruct, const int32_t* n_atoms, const double* pos,
                     const double* velo, const double* mass, const int32_t* Z, const double* lattices,
                     const int32_t* pbcs, double dt, double skin, gapgpu_md** out);
int gapgpu_md_step(gapgpu_md* md, int nsteps);
/* Current positions, velocities, forces (nullable host arrays) and per-replica
 * potential energies and virials. */
int gapgpu_md_state(gapgpu_md* md, double* pos, double* velo, double* force, double* energies, double* virials);
int gapgpu_md_counters(const gapgpu_md* md, int64_t* steps, int64_t* rebuilds, int64_t* graph_replays);
gapgpu_context* gapgpu_md_context(gapgpu_md* md);
void gapgpu_md_destroy(gapgpu_md* md);

/* Failure-detection self-test: a kernel waits on a device barrier that is never
 * signalled, with the bounded wait the tensor-core GEMMs use (which give up after 250 ms
 * of GPU time), here limit_us microseconds long (1..10^6).  Returns GAPGPU_ERR_TIMEOUT with
 * a message once the wait has given up; the context stays usable.  Used by the tests; no
 * counterpart in the reference. */
int gapgpu_selftest_bounded_wait(gapgpu_context* ctx, int64_t limit_us);

/* Diagnostic: the FP32 FMA rate of this GPU in TFLOP/s (2 FLOP per FMA), measured with
 * CUDA events on the context's stream by an FMA-loop kernel, scalar and packed (f32x2)
 * FMAs, the larger of the two.  The ceiling against which the SIMT kernels' rates are
 * reported; no counterpart in the reference. */
int gapgpu_probe_fp32_rate(gapgpu_context* ctx, double* tflops);

/* Wait for the context's stream. */
int gapgpu_context_sync(gapgpu_context* ctx);

/* LAMMPS pair_style quip path: quip_lammps_wrapper (src/Potentials/quip_lammps_wrapper.f95:
 * 30-156) with the host's own neighbour list and explicit ghost atoms (no periodic
 * shifts; `lattice` only enters the virial's bookkeeping).  nlocal + nghost atoms with
 * Z and pos double[3*(nlocal+nghost)]; ilist[inum] (0-based) lists the local atoms,
 * which are the only centres (atom_mask_name=local); num_neigh[inum] and neigh (packed,
 * 1-based, as the wrapper reads them) give each local atom's FULL neighbour list.
 * Outputs (nullable) have the wrapper's shapes: energy, local_e[n], virial[9],
 * local_virial[9n], force[3n] including the forces on ghosts, which the host sums back
 * onto their owners.  Uses the context's precision. */
int gapgpu_calc_lammps(gapgpu_context* ctx, int nlocal, int nghost, const int32_t* Z, int inum, const int32_t* ilist,
                       const int32_t* num_neigh, const int32_t* neigh, const double* lattice, const double* pos,
                       double* energy, double* local_e, double* virial, double* local_virial, double* force);

/* Neighbour list with QUIP semantics (no minimum image, every periodic image within
 * `cutoff`, strict r < cutoff) built on the GPU: connection_calc_connect
 * (Connection.f95:1035-1310).  Returns per-atom CSR (offsets n+1, j, shift 3 per
 * entry); when `capacity` is too small only offsets/total are filled.  Order within an
 * atom's list is deterministic but not the reference's linked-list order. */
int gapgpu_neighbours(gapgpu_context* ctx, int n, const double* pos, const double* lattice, const int32_t* pbc,
                      double cutoff, int32_t* offsets, int32_t* nbr_j, int32_t* nbr_shift, int64_t capacity,
                      int64_t* total);

/* Largest structure gapgpu_neighbours_static accepts. */
#define GAPGPU_STATIC_MAX_ATOMS 65536

/* gapgpu_neighbours_static: the neighbour list of gapgpu_neighbours for callers that
 * cannot allocate GPU memory.  It has no counterpart in the reference.
 *
 * Who needs it: host codes whose device memory all belongs to their own pool allocator
 * (an MD engine's memory space, a framework that reserves most of HBM at start-up), and
 * time-step loops that must not call cudaMalloc/cudaFree, which synchronise the device
 * and stall the host code's other streams.  This entry point makes no allocation:
 * no cudaMalloc, no cudaFree and no allocating library routine.  Its scratch lives in one
 * fixed device array of about 9 MiB, which every GPU that loads the library holds until
 * the process exits.
 *
 * The caller owns every input and output, all device pointers except lattice, pbc and
 * total: d_pos double[3n] (Fortran pos(3,N)), d_offsets int32[n+1], d_nbr_j
 * int32[capacity], d_nbr_shift int32[3*capacity] (same layout as gapgpu_neighbours).
 * *total receives the number of entries; when capacity < *total, or d_nbr_j or
 * d_nbr_shift is NULL, only d_offsets and *total are written.  Atoms that overlap
 * exactly (a pair distance below 1e-10, GAPGPU_ERR_ATOMS) are detected only by a call
 * that fills the list: a count-only call returns GAPGPU_OK with offsets for such a
 * structure, and the error comes from the second call of the count-then-fill pattern.
 * The work runs on cuda_stream (NULL = the legacy default stream), and the call waits
 * for that stream and copies the count to the host before it returns, so no call of it
 * can be made while cuda_stream is being captured into a CUDA graph.
 *
 * Limits: n <= GAPGPU_STATIC_MAX_ATOMS (GAPGPU_ERR_ARG above it).  The scratch array is
 * shared by every call in the process and keeps the previous call's contents, so calls
 * that overlap on the GPU (other host threads, other streams) race: serialise them.
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress), with that device current. */
int gapgpu_neighbours_static(int n, const double* d_pos, const double* lattice, const int32_t* pbc, double cutoff,
                             int32_t* d_offsets, int32_t* d_nbr_j, int32_t* d_nbr_shift, int64_t capacity,
                             int64_t* total, void* cuda_stream);

/* The neighbour list a context holds after its last evaluation or MD step -- the
 * connection at%connect after calc_connect or, when the list was kept on its skin,
 * after connection_calc_dists refreshed it (Connection.f95:1086-1125, :1321-1445) --
 * read back without rebuilding: per-atom CSR over the evaluation's atoms (structures
 * of a batch or MD replicas concatenated, indices global), j, shift (3 per entry) and
 * the distance r of each entry.  A list kept on a skin holds every pair within
 * cutoff + skin.  When capacity is too small only offsets and *total are written. */
int gapgpu_context_neighbours(gapgpu_context* ctx, int32_t* offsets, int32_t* nbr_j, int32_t* nbr_shift, double* nbr_r,
                              int64_t capacity, int64_t* total);

/* SOAP descriptors (and the sum of squares before normalisation) of every centre
 * for coordinate `coordinate` of the model: the descriptor-only path of
 * quippy/quippy/descriptors.py:165-235.  q: n_centres*dim row-major. */
int gapgpu_descriptors(gapgpu_context* ctx, int coordinate, int n, const double* pos, const int32_t* Z,
                       const double* lattice, const int32_t* pbc, double* q, int64_t capacity, int* n_centres);

/* Last calculation's stage timings in ms (CUDA events): neighbours, soap_fwd, gemm,
 * soap_bwd, pair2b, reduce, total.  Returns the number of entries written. */
int gapgpu_context_timings(const gapgpu_context* ctx, double* ms, int capacity);

/* Number of this library's kernel launches issued by the last calculation. */
int gapgpu_context_launches(const gapgpu_context* ctx, int64_t* launches);

#ifdef __cplusplus
}
#endif
#endif /* GAPGPU_H */
