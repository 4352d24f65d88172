/*
 * ephg.h - C ABI of the GB300 (sm_103a) e-ph vertex library.
 *
 * Drop-in for elphbolt's Wannier-interpolation procedures and the electron-
 * and phonon-side e-ph rate drivers, callable from Fortran through ISO_C_BINDING
 * (the bind(C) interfaces are in include/wannier_gpu.f90).  Every entry point names
 * the reference procedure it replaces.
 *
 * Conventions
 *  - Arrays are caller-owned, Fortran column-major, with the reference's
 *    shapes; complex(r64) arrays are interleaved (re, im) doubles.
 *  - Sizes are int64_t; integer indices that the reference keeps 1-based
 *    (muxed wave-vector indices, band indices) stay 1-based.
 *  - Every call returns EPHG_OK (0) or an error code; ephg_last_error() gives
 *    the message of the calling thread's last failure.  Where the reference
 *    stops the program (exit_with_message, src/misc.f90:194-203) the library
 *    returns the matching code instead.
 *  - The handle owns all device memory; one handle per host thread.
 */
#ifndef EPHG_H
#define EPHG_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EPHG_OK 0
#define EPHG_ERR_ARG 1            /* invalid argument */
#define EPHG_ERR_CUDA 2           /* CUDA runtime error or no device */
#define EPHG_ERR_NEG_PHONON 3     /* "Large negative phonon energy found!" wannier.f90:775 */
#define EPHG_ERR_EMPTY_WINDOW 4   /* "No states found within Fermi window." electron.f90:627 */
#define EPHG_ERR_EIG 5            /* Jacobi eigensolver did not converge */
#define EPHG_ERR_NOMEM 6          /* device memory budget exceeded */
#define EPHG_ERR_TIMEOUT 7        /* a bounded device wait gave up */
#define EPHG_ERR_INDEX 8          /* device-side index check failed */

#define EPHG_PREC_FP64 0          /* plain FP64 drop-in */
#define EPHG_PREC_SPLIT_TF32 1    /* 3xTF32 tcgen05 contractions, FP32 accumulate */

#define EPHG_DELTA_GAUSSIAN 0     /* fixed-sigma Gaussian / N_k */
#define EPHG_DELTA_TRIANGLE 1     /* delta_fn_triang, src/delta.f90:790 */
#define EPHG_DELTA_TETRA 2        /* delta_fn_tetra,  src/delta.f90:61 */

#define EPHG_WANNSPACE_EL 0
#define EPHG_WANNSPACE_PH 1

typedef struct ephg_handle ephg_handle;

/* Real-space Wannier data: the fields of type Wannier (src/wannier.f90:46-93)
 * plus the crystal data the path reads (src/crystal.f90). */
typedef struct {
  int64_t numwannbands;       /* nw */
  int64_t numbranches;        /* nb = 3 * numatoms */
  int64_t nwsk, nwsq, nwsg;   /* WS cell counts; nwsg must equal nwsq (wannier.f90:947) */
  int64_t numatoms;
  int64_t coarse_qmesh[3];
  const double *lattvecs;     /* (3,3) nm, columns a1 a2 a3 */
  const double *basis;        /* (3,numatoms) crystal coordinates */
  const double *masses;       /* (numatoms) amu, masses(atomtypes(i)) */
  const int64_t *rcells_k;    /* (nwsk,3) */
  const int64_t *rcells_q;    /* (nwsq,3) */
  const int64_t *rcells_g;    /* (nwsg,3) */
  const int64_t *elwsdeg;     /* (nwsk) */
  const int64_t *phwsdeg;     /* (nwsq) */
  const int64_t *gwsdeg;      /* (nwsg) */
  const double *Hwann;        /* complex (nwsk,nw,nw), Ry */
  const double *Dphwann;      /* complex (nwsq,nb,nb), Ry/bohr^2 */
  const double *gwann;        /* complex (nw,nw,nwsk,nb,nwsg), Ry/bohr, epmatwp order */
} ephg_wannier_desc;

/* One electron RTA-rate request (the numerics/electron settings the
 * ibzk driver reads: mesh, enref, fsthick, chempot, T, delta method). */
typedef struct {
  int64_t mesh[3];            /* electron mesh = phonon mesh (mesh_ref = 1) */
  double enref;               /* eV, window centre */
  double fsthick;             /* eV, window half width */
  double chempot;             /* eV */
  double T;                   /* K */
  int64_t delta_kind;         /* EPHG_DELTA_* */
  double sigma;               /* eV, Gaussian width */
  int64_t precision;          /* EPHG_PREC_* */
} ephg_rate_request;

typedef struct {
  int64_t nwv;                /* window k-points (FBZ blocks = IBZ blocks) */
  int64_t nstates_inwindow;   /* window (k', n) final states */
  int64_t nstates;            /* window initial states (k, m) */
  int64_t vertices;           /* |g|^2 vertices, the count of interactions.f90:2261 */
  int64_t pairs;              /* (initial state, k') pairs */
  int64_t kernel_launches;    /* library kernels launched by the call */
  double ms_setup;            /* H(k), D(q), eigensolves, window, tables */
  double ms_stage_a;          /* g(Re,Rp) -> g(k,Rp) and the initial-band rotation */
  double ms_stage_bc;         /* Rp Fourier + rotations + |g|^2 + delta + rates */
  double ms_total;            /* device time of the whole call */
  double stage_b_gflop;       /* algorithmic GFLOP of the Rp Fourier contraction */
  double stage_a_gflop;       /* algorithmic GFLOP of the Re contraction */
  double ms_gemm_a;           /* summed device time of the stage-A contraction launches */
  double ms_gemm_b;           /* summed device time of the stage-B contraction launches */
  int64_t gemm_a_launches;
  int64_t gemm_b_launches;
} ephg_rate_stats;

/* Upload the Wannier data once; the returned handle keeps it resident in HBM
 * (replaces Wannier%read, wannier.f90:97-140, and read_EPW_Wannier :289). */
int ephg_create(const ephg_wannier_desc *desc, ephg_handle **out);
int ephg_destroy(ephg_handle *h);
const char *ephg_last_error(void);
/* Number of CUDA devices visible (0 on a machine without a GPU). */
int ephg_device_count(void);
/* The library keeps device memory freed by ephg_destroy and by released
 * workspaces mapped in a pool of its own (up to half the device), so that the
 * next handle or request reuses it at no cost.  This returns the pool's unused
 * memory on the current device to the driver, for a caller that needs it for
 * other allocations; memory of live handles is untouched. */
int ephg_trim_memory(void);

/* The crystal fields of a polar crystal (crys%polar = .true.; crystal.f90:45-49):
 * epsilon (3,3) the high-frequency dielectric tensor and born (3,3,numatoms)
 * the Born effective charges, born(:, ipol, iat) as the reference reads them.
 * From then on ph_wann adds dyn_nonanalytic (wannier.f90:784-901) to D(q) and
 * every |g|^2 (g2, el_rates, ph_rates) adds long_range_prefac (:1013-1071)
 * times the electron overlap (:998-1006).  epsilon NULL: non-polar again. */
int ephg_set_polar(ephg_handle *h, const double *epsilon, const double *born);

/* Crystal symmetry (symmetry.f90).
 *
 * ephg_crystal_symmetry: the space-group operations of a crystal, what
 * spg_get_dataset gives calculate_symmetries (symmetry.f90:66-110) with the
 * tolerance symprec (nm): x' = W x + t in crystal coordinates, rotations
 * (3,3,nops) column-major integer W, translations (3,nops); lattvecs (3,3)
 * columns a1 a2 a3 (nm), basis (3,natoms) crystal coordinates, atomtypes
 * (natoms).  The identity comes first; the other operations in a fixed order
 * of this library (spglib's order may differ).  maxops: room in the outputs.
 *
 * ephg_set_symmetry: the nsymm real-space rotations (3,3,nsymm) of the crystal
 * (rotations_orig; NULL / 0: the identity only).  Every rate request then
 * forms, per its mesh, the reciprocal rotations with time reversal, without
 * those incompatible with the mesh or repeated (symmetry.f90:134-212), and
 * - gives every mesh point the electron energies of its irreducible point
 *   (electron.f90:363-385, 531-546; the eigenvectors stay the point's own);
 * - ephg_el_rates takes initial states on the irreducible window points only
 *   (IBZ blocks, electron.f90:553-577; interactions.f90:2169-2191): rates and
 *   indexlist have stats.nwv rows, one per irreducible window point, in
 *   indexlist_irred order -- rta_rates_eph(nwv_irred, nw);
 * - ephg_ph_rates keeps every window k (the phonon side sums over them) and
 *   returns every q of the mesh.
 *
 * ephg_irred_wedge: find_irred_wedge (symmetry.f90:303-452) with the nsymm
 * real-space rotations of a lattice (as for ephg_set_symmetry; no device is
 * needed) on a mesh, over its nk points of indexlist (1-based muxed, sorted;
 * NULL: the whole mesh): nirred irreducible points indexlist_irred, their
 * nequiv images and fbz2ibz (nk, nullable) the 1-based irreducible point of
 * every input point (create_fbz2ibz_map, :480-503).  Outputs sized nk. */
int ephg_crystal_symmetry(const double *lattvecs, int64_t natoms, const double *basis, const int64_t *atomtypes,
                          double symprec, int64_t maxops, int64_t *nops, int64_t *rotations, double *translations);
int ephg_set_symmetry(ephg_handle *h, int64_t nsymm, const int64_t *rotations);
int ephg_irred_wedge(const double *lattvecs, int64_t nsymm, const int64_t *rotations, const int64_t mesh[3],
                     int64_t nk, const int64_t *indexlist, int64_t *nirred, int64_t *indexlist_irred, int64_t *nequiv,
                     int64_t *fbz2ibz);

/* el_wann (wannier.f90:430-524): kvecs (nk,3) crystal coords -> energies
 * (nk,nw) eV; optional velocities (nk,nw,3) km/s, evecs (nk,nw,nw) with
 * evecs(k,b,:) the eigenvector of band b, scissor (nw) eV.  NULL = absent. */
int ephg_el_wann(ephg_handle *h, int64_t nk, const double *kvecs, double *energies,
                 double *velocities, double *evecs, const double *scissor);

/* ph_wann, non-polar (wannier.f90:585-782): qvecs (nq,3) -> energies (nq,nb) eV,
 * optional evecs (nq,nb,nb) with evecs(q,s,:) the eigenvector of mode s,
 * velocities (nq,nb,3) km/s.  Returns EPHG_ERR_NEG_PHONON where the reference stops. */
int ephg_ph_wann(ephg_handle *h, int64_t nq, const double *qvecs, double *energies,
                 double *evecs, double *velocities);

/* gkRp (wannier.f90:1073-1132), batched over k: gmixed (nw,nw,nb,nwsq,nk). */
int ephg_gkRp(ephg_handle *h, int64_t nk, const double *kvecs, double *gmixed);

/* gReq (wannier.f90:1134-1188), batched over q: gmixed (nw,nw,nb,nwsk,nq). */
int ephg_gReq(ephg_handle *h, int64_t nq, const double *qvecs, double *gmixed);

/* g2 (wannier.f90:903-1011, non-polar), batched over vertices.  Vertex v uses
 * gmixed(:,:,:,:,gm_index(v)) (1-based) of the ngm blocks passed, with nws =
 * nwsg cells for wannspace PH and nwsk for EL.  Arrays: kvecs, qvecs (nv,3);
 * el_evec_k, el_evec_kp (nv,nw) complex; ph_evec_q (nv,nb) complex; ph_en (nv). */
int ephg_g2(ephg_handle *h, int64_t wannspace, int64_t nv, const double *kvecs,
            const double *qvecs, const double *el_evec_k, const double *el_evec_kp,
            const double *ph_evec_q, const double *ph_en, int64_t ngm, const double *gmixed,
            const int64_t *gm_index, double *g2_out);

/* vector_allreps_sub (src/vector.f90:86-102) batched on the device:
 * q(i,j) = muxed index of k'(j) - k(i) folded onto the mesh, all 1-based.
 * k_idx (nk), kp_idx (nkp) muxed indices; q_idx (nk,nkp). */
int ephg_kq_index(ephg_handle *h, const int64_t mesh[3], int64_t nk, const int64_t *k_idx,
                  int64_t nkp, const int64_t *kp_idx, int64_t *q_idx);

/* calculate_eph_interaction_ibzk 'g' + 'X' (interactions.f90:2095-2400) fused
 * with calculate_el_rta_rates (interactions.f90:2958-3063), identity point
 * group, q mesh = k mesh, no disk.  rates (N_k,nw) column-major with the first
 * stats.nwv rows valid (window k order = indexlist order); indexlist (N_k)
 * receives the window's muxed indices.  Optional per-vertex outputs in the
 * reference's order (initial state, k', n, s) with capacity cap: g2 (eV^2),
 * xplus, xminus (THz).  stats may be NULL. */
int ephg_el_rates(ephg_handle *h, const ephg_rate_request *req, double *rates,
                  int64_t *indexlist, ephg_rate_stats *stats, double *g2, double *xplus,
                  double *xminus, int64_t cap);

/* ephg_el_rates for nsets requests (1 <= nsets <= EPHG_MAX_SETS) that differ
 * only in T, sigma and chempot: mesh, window (enref, fsthick), delta_kind
 * and precision equal, else EPHG_ERR_ARG.  The vertices and |g|^2 depend on
 * none of the three, so the contractions run once and the rate epilogue once
 * per set: rates[i] (N_k,nw) receives what ephg_el_rates returns for reqs[i];
 * indexlist and stats (nullable; stats counts one set's vertices) are common.
 * The reference takes one temperature and chemical potential per run
 * (input.nml); a sweep over them there is one run per point. */
#define EPHG_MAX_SETS 8
int ephg_el_rates_sets(ephg_handle *h, int64_t nsets, const ephg_rate_request *reqs, double *const *rates,
                       int64_t *indexlist, ephg_rate_stats *stats);

/* calculate_eph_interaction_ibzq 'g' + 'Y' (interactions.f90:1673-1930, the 'Y'
 * pass as calculate_Y_OTF :1932-2093) fused with the ph-e part of
 * calculate_ph_rta_rates (interactions.f90:2723-2828), identity point group,
 * q mesh = k mesh, no disk.  rates_phe (N_q,nb) column-major: row iq - 1 is
 * the phonon of muxed q index iq (every q of the mesh: the phonon side has no
 * window); spindeg is el%spindeg, 1 or 2 (electron.f90:164).  The vertices are
 * those of ephg_el_rates -- vertex (k, m, k + q, n, s) of phonon state (q, s) is
 * vertex (k, m, k', n, s) of the electron side with k' = k + q -- so one sweep
 * forms both sides: el_rates (N_k,nw) and indexlist (N_k), if not NULL,
 * receive what ephg_el_rates returns.  Optional per-vertex lists in the order
 * of ephg_el_rates, capacity cap: g2 (eV^2) and y (Y in THz, before the
 * spindeg factor).  stats may be NULL. */
int ephg_ph_rates(ephg_handle *h, const ephg_rate_request *req, int64_t spindeg, double *rates_phe,
                  double *el_rates, int64_t *indexlist, ephg_rate_stats *stats, double *g2, double *y,
                  int64_t cap);

/* Degenerate-subspace gauge fixing of |g|^2 (plot_along_path, wannier.f90:
 * 1332-1384; the same loops in test/check_interactions_symmetries.f90:330-384),
 * FP64 on the device.  g2 (nv): a vertex list of req in the order
 * ephg_el_rates writes it (every vertex: nv = stats.vertices, either
 * precision, or read back from gk2.istate files), replaced in place.  Three
 * passes in the reference's order: over the phonon branches s of q = k' - k
 * (|omega_s - omega_s'| < thres), the initial bands m of each k and the final
 * bands n of each k' (|E - E'| < thres); thres in eV (<= 0: the reference's
 * 1e-6).  The band groups are the window bands, the only ones the list holds.
 * mode EPHG_DEGAVG_REFERENCE: the reference's loops as written, in place -- a
 * member averages values its predecessors in the group have already replaced,
 * so its result still depends on the eigenvector gauge; EPHG_DEGAVG_MEAN:
 * every member takes the mean of the group's values before the pass, which is
 * gauge invariant.  Runs the request's set-up (energies, phonons, window), not
 * its contractions.  The reference's rate path does not average; nor does
 * ephg_el_rates. */
#define EPHG_DEGAVG_REFERENCE 0
#define EPHG_DEGAVG_MEAN 1
int ephg_g2_average_degenerate(ephg_handle *h, const ephg_rate_request *req, int64_t mode, double thres,
                               int64_t nv, double *g2);

/* ---- Serving loop ----
 * No counterpart in the reference, which answers one request per run from
 * disk; this is the scope's serving form.  A server keeps the crystals of
 * `crystals` (handles of ephg_create, on one device, which must outlive it and
 * must not be used directly while it runs) resident and answers RTA-rate
 * requests as they arrive, by continuous batching: it owns nslots execution
 * slots (a stream, a request workspace and timers each); a free slot takes the
 * oldest waiting request at once, and the requests of different slots run
 * concurrently on the device.  A served result equals the same request run
 * alone (ephg_el_rates).  Admission is by an HBM budget covering the crystals'
 * resident data and the slots' workspaces, an equal share per slot:
 * ephg_submit refuses (EPHG_ERR_NOMEM) a request whose set-up arrays alone
 * cannot fit; a request that does not fit its slot's share waits for the other
 * slots to go idle (no new request starts meanwhile), takes the whole budget,
 * and fails with EPHG_ERR_NOMEM before allocating only if that is still too
 * little.  A free slot takes the waiting request of highest response ratio
 * (its age over its estimated isolated solve time, from a per-crystal fit of
 * the solve times seen), with the queued requests that can share its
 * contraction (ephg_server_set_merge); a request much smaller than a running
 * one runs on a high-priority stream, and served requests run their persistent
 * kernels as launches of a few ms, between which the GPU goes to the running
 * request of highest ratio.  Latency is the wall time from ephg_submit to
 * completion. */
typedef struct ephg_server ephg_server;

#define EPHG_TICKET_QUEUED 0
#define EPHG_TICKET_RUNNING 1
#define EPHG_TICKET_DONE 2
#define EPHG_TICKET_FAILED 3

typedef struct {
  int64_t submitted, completed, failed, rejected;
  int64_t vertices;             /* |g|^2 vertices of the completed requests */
  double p50_ms, p99_ms, max_ms, mean_ms;   /* submit -> completion, completed requests (nearest rank) */
  double wall_s;                /* first submit -> last completion */
  double vertices_per_s;        /* vertices / wall_s */
  int64_t peak_device_bytes;    /* largest resident + workspace total seen after a request */
  int64_t merged;               /* completed requests that shared another request's contraction */
} ephg_server_stats;

int ephg_server_create(ephg_handle *const *crystals, int ncrystals, int64_t hbm_budget_bytes, int nslots,
                       ephg_server **out);
/* Stops the worker after the running request; queued requests fail. */
int ephg_server_destroy(ephg_server *s);
/* Queue a request for crystal index `crystal`; returns at once with a ticket. */
int ephg_submit(ephg_server *s, int crystal, const ephg_rate_request *req, int64_t *ticket);
/* Non-blocking: *state = EPHG_TICKET_QUEUED / RUNNING / DONE / FAILED. */
int ephg_poll(ephg_server *s, int64_t ticket, int *state);
/* Block until the ticket completes, then copy its results (buffers sized as
 * for ephg_el_rates: rates (N,nw), indexlist (N), N = mesh points) and its
 * latency (submit -> completion, ms), and retire the ticket; any output may
 * be NULL.  Returns the request's status. */
int ephg_wait(ephg_server *s, int64_t ticket, double *rates, int64_t *indexlist, ephg_rate_stats *stats,
              double *latency_ms);
int ephg_server_stats_get(ephg_server *s, ephg_server_stats *out);
/* Merging (default EPHG_MAX_SETS): a free slot that takes a request also
 * takes, up to max_sets in all, the queued requests of the same crystal that
 * differ from it only in T, sigma and chempot, and runs them as one
 * ephg_el_rates_sets call (one contraction, an epilogue per request); each
 * result still equals its request run alone.  max_sets = 1 turns it off. */
int ephg_server_set_merge(ephg_server *s, int max_sets);

/* ---- Batched form ----
 * No counterpart in the reference (one crystal, one request per run).  n rate
 * requests, request i against crystal handle crystals[i] (any number of
 * distinct handles, repeats allowed), solved together: up to nslots requests
 * run at once, one host thread and stream each, largest estimated work first.
 * With grouped != 0 the split form's generic contractions (every shape but
 * the nw = 8, nb = 6 Gaussian one, which runs its own fused kernels) meet in
 * rounds: when every request inside a contraction stage has reached its next
 * GEMM, those GEMMs (different crystals, shapes and operands) run as ONE
 * persistent tcgen05 launch over all their tiles.  The requests' workspaces
 * share hbm_budget_bytes (0: 80% of the device memory free at the call); a
 * request that does not fit runs again alone after the others, with the
 * whole budget.  Outputs per request as for ephg_el_rates (rates[i] (N_i,nw_i),
 * indexlists[i] (N_i), stats + 0..n-1 nullable), status[i] its return code;
 * every result equals the same request run alone.  Returns EPHG_OK when every
 * request succeeded, else the first failing request's code. */
typedef struct {
  int64_t nslots;             /* requests running at once, 1..64; 0 = 8 */
  int64_t hbm_budget_bytes;   /* workspace budget of the batch; 0 = 80% of the free device memory */
  int64_t grouped;            /* 1: grouped GEMM launches across the running requests; 0: each its own */
} ephg_batch_opts;

typedef struct {
  int64_t requests, failed, vertices;
  double wall_ms;             /* host wall time of the call */
  double vertices_per_s;      /* vertices / wall_ms */
  int64_t group_launches;     /* grouped GEMM launches */
  int64_t group_problems;     /* GEMMs they ran */
  int64_t group_tiles;        /* 128 x 128 output tiles they ran */
  int64_t max_group;          /* most GEMMs in one launch */
  int64_t retried_alone;      /* requests re-run alone after their workspace did not fit */
  int64_t peak_workspace_bytes;
} ephg_batch_stats;

int ephg_el_rates_batch(int64_t n, ephg_handle *const *crystals, const ephg_rate_request *reqs,
                        double *const *rates, int64_t *const *indexlists, ephg_rate_stats *stats, int *status,
                        const ephg_batch_opts *opts, ephg_batch_stats *bstats);

/* el_wann without any device allocation.  No counterpart in the reference:
 * it serves callers that cannot allocate device memory where they need the
 * electrons -- a host code handing over buffers it already owns on the device
 * (OpenACC or CUDA Fortran arrays, or system memory the GPU reaches over the
 * Grace C2C link), a process whose device memory is fixed by another
 * framework's pool, or a time-critical loop that must not pay cudaMalloc's
 * implicit synchronisation.  kvecs (nk,3) is read and energies (nk,nw) and
 * evecs (nk,nw,nw, nullable) written through the caller's device-accessible
 * pointers, in the layouts of ephg_el_wann (no velocities, no scissor).  The
 * scratch is one fixed array of EPHG_NOALLOC_SCRATCH_BYTES inside the library
 * (every GPU that loads the library holds it until exit); requests that need
 * more are refused with EPHG_ERR_ARG and the largest nk that fits in the
 * message.  The first call on a device resolves the array's address (set-up),
 * so make it before any stream capture; later calls outside a capture resolve
 * it again (a re-created context is picked up).  All calls share the array:
 * calls that overlap on the GPU race.  The handle's device must be current.
 * The kernels run on the handle's own stream, which does not wait for other
 * streams: kvecs must be complete before the call (synchronise the stream or
 * OpenACC queue that wrote it), and the call returns after the handle's stream
 * has finished, so energies and evecs are complete on return. */
#define EPHG_NOALLOC_SCRATCH_BYTES (16ull << 20)
int ephg_el_wann_noalloc(ephg_handle *h, int64_t nk, const double *kvecs, double *energies,
                         double *evecs);

#ifdef __cplusplus
}
#endif
#endif
