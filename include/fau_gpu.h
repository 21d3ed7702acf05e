/*
 * fau_gpu.h -- C ABI of the GB300 Metropolis Monte Carlo energy hot path.
 *
 * The library replaces, for one process on one GPU, the part of Faunus that
 * runs once per trial move:
 *
 *   MetropolisMonteCarlo::performMove        src/montecarlo.cpp:139-187
 *     Hamiltonian::updateState / energy       src/energy.cpp:1227-1252
 *       Nonbonded<...>::energy                src/energy.h:1561-1577
 *       Ewald::updateState / energy           src/energy.cpp:564-587
 *     getEnergyChange                         src/montecarlo.cpp:193-209
 *     metropolisCriterion                     src/montecarlo.cpp:17-34
 *     State::sync (accept / reject)           src/montecarlo.cpp:250-254
 *
 * Conventions (no exceptions cross this boundary):
 *   - every entry point returns an int status (FAU_OK == 0);
 *     fau_strerror() names it and fau_last_error() gives the detail text
 *     of the last failure on the calling thread;
 *   - handles are opaque; all pointers in descriptors are HOST pointers to
 *     caller-owned memory that is only read during the call;
 *   - energies are in kT at the system temperature, lengths in angstrom;
 *   - one host thread per context: calls on the same context are serialised
 *     by the caller (the reference is single threaded per process).
 */
#ifndef FAU_GPU_H
#define FAU_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FAU_ABI_VERSION 1

/* ---- status codes -------------------------------------------------------- */
enum fau_status {
    FAU_OK = 0,
    FAU_ERR_ARG = 1,       /* invalid argument or unsupported combination       */
    FAU_ERR_OOM = 2,       /* device allocation or HBM budget exceeded          */
    FAU_ERR_CUDA = 3,      /* CUDA runtime error (detail in fau_last_error)     */
    FAU_ERR_TIMEOUT = 4,   /* a bounded device wait ran out                     */
    FAU_ERR_NAN = 5,       /* NaN energy change: metropolisCriterion throws     */
    FAU_ERR_CAPACITY = 6,  /* a device cell-list cell overflowed                */
    FAU_ERR_STATE = 7,     /* call not valid in the handle's current state      */
    FAU_ERR_NODEVICE = 8   /* no CUDA device / driver                           */
};

/* ---- pair potential composition ------------------------------------------
 * A pair energy is the sum of the enabled terms, as the reference's
 * CombinedPairPotential (src/potentials_base.h:226-286) and
 * FunctorPotential compositions (src/potentials.h:728-755).               */
enum fau_pair_term {
    FAU_PAIR_COULOMB = 1 << 0, /* lB qi qj S(r) / r                             */
    FAU_PAIR_LJ = 1 << 1,      /* 4 eps [(s/r)^12 - (s/r)^6]   potentials.h:42-49  */
    FAU_PAIR_WCA = 1 << 2,     /* LJ + eps, zero beyond 2^(1/6) s   :151-160     */
    FAU_PAIR_HS = 1 << 3,      /* +inf when r < s                   :203-207     */
    FAU_PAIR_SPLINE = 1 << 4   /* nonbonded_splined: the sum of the terms above
                                  tabulated per atom-type pair (spline_* below;
                                  SplinedPotential src/potentials.h:770-824)      */
};

/* Coulomb short-range function S(q = r/Rc) (docs/_docs/energy.md:169-205). */
enum fau_coulomb_type {
    FAU_COUL_PLAIN = 0, /* S = 1, no cutoff  (Coulomb potentials.h:472-476)        */
    FAU_COUL_CUT = 1,   /* S = 1 for r < Rc, 0 beyond (poisson C=1, D=-1)         */
    FAU_COUL_EWALD = 2, /* S = erfc(alpha r) for r < Rc, 0 beyond (kappa = 0)      */
    FAU_COUL_TRUNC = 3  /* S = e erfc(alpha r) + sum_k c_k q^k for r < Rc, 0 beyond:
                           reactionfield, poisson, qpotential, fanourgakis, fennell,
                           zerodipole, zahn, wolf at kappa = 0 (coulomb_poly below) */
};
#define FAU_COUL_MAX_POLY 16

/* group flags: MoleculeData::atomic / rigid (src/molecule.h:222-279) */
enum fau_group_flag {
    FAU_GROUP_ATOMIC = 1 << 0,
    FAU_GROUP_RIGID = 1 << 1
};

/* arithmetic of the dU evaluation */
enum fau_precision {
    FAU_PREC_FP32C = 0, /* FP32 pair/Ewald terms, compensated sums, FP64 totals */
    FAU_PREC_FP64 = 1   /* plain FP64 evaluation: one move per call in the
                           single-system calls (the in-GPU comparison form),
                           persistent FP64 chains in the batch calls          */
};

/* Ewald reciprocal space, EwaldData (src/energy.cpp:28-59), PBC policy. */
typedef struct fau_ewald_desc {
    int enabled;       /* 1: add Ewald reciprocal + surface terms             */
    double alpha;      /* damping parameter (1/angstrom)                      */
    double ncutoff;    /* reciprocal cutoff in units of 2 pi / L               */
    int spherical_sum; /* 1: keep only n^2 <= ncutoff^2                        */
    double epss;       /* surface dielectric constant; < 1 means tinfoil      */
} fau_ewald_desc;

/* A Space + Hamiltonian pair as the reference builds it from its input. */
typedef struct fau_sys_desc {
    int n_particles;
    double box[3];            /* cuboid side lengths                                */
    const double* pos;        /* n*3 xyz, each inside [-L/2, L/2] (Particle::pos)   */
    const double* charge;     /* n (Particle::charge)                                */
    const int* type;          /* n atom type ids in [0, n_types) (Particle::id)      */

    int n_groups;
    const int* group_begin;   /* n_groups + 1 offsets into the particle arrays       */
    const int* group_molid;   /* n_groups molecule ids                               */
    const int* group_flags;   /* n_groups fau_group_flag bits                        */
    const double* group_mass_center; /* n_groups*3 Group::mass_center; NULL: computed */

    int n_types;
    const double* type_mass;  /* n_types AtomData::mw (mass centres); NULL: all 1    */
    const double* sigma2;     /* n_types^2 LJ/WCA sigma_ij^2                         */
    const double* eps4;       /* n_types^2 LJ/WCA 4 eps_ij in kT                     */
    const double* hs_sigma2;  /* n_types^2 hard-sphere sigma_ij^2                    */

    int pair_terms;           /* fau_pair_term bits                                  */
    int coulomb_type;         /* fau_coulomb_type                                    */
    double bjerrum_length;    /* lB (angstrom)                                       */
    double coulomb_cutoff;    /* Rc of FAU_COUL_CUT / FAU_COUL_EWALD                 */
    double coulomb_alpha;     /* alpha of FAU_COUL_EWALD real space                  */
    double pair_cutoff;       /* > 0: every pair term is zero beyond this distance
                                 and the device uses cell lists for single-atom
                                 moves; <= 0: all pairs, reference semantics        */
    double cutoff_g2g;        /* GroupCutoff mass-centre cutoff; <= 0: none          */
    fau_ewald_desc ewald;

    int precision;            /* fau_precision                                       */
    int cell_capacity;        /* slots per cell; 0: chosen from the initial state    */
    int n_molids;             /* molecule kinds (group_molid < n_molids) of the matrix below */
    const double* cutoff_g2g_pairs; /* n_molids^2 GroupCutoff::getCutoff(i, j) per molecule-kind
                                 pair (src/energy.h:746-768); <= 0 or +inf: no cutoff for
                                 that pair; NULL: cutoff_g2g for every pair                */
    /* FAU_COUL_TRUNC: S(q) = coulomb_erfc * erfc(coulomb_alpha r) + sum_{k < coulomb_poly_n}
       coulomb_poly[k] q^k, q = r / coulomb_cutoff; self energy lB q_i^2 S'(0) / (2 Rc)  */
    int coulomb_poly_n;
    double coulomb_erfc;
    double coulomb_poly[FAU_COUL_MAX_POLY];
    int isobaric;             /* 1: the Hamiltonian has the Isobaric term (src/energy.cpp:859-901) */
    double pressure;          /* its pressure in kT / A^3                             */
    /* FAU_PAIR_SPLINE: per atom-type pair ab = a * n_types + b, Andrea spline knots z_0 < ... <
       z_m in r^2 with 6 coefficients an interval (KnotData, src/potentials.h:773-780; made by
       fau_spline_tabulate). SplinedPotential::operator() (src/potentials.h:807-823): 0 for
       r^2 >= z_m; sum_k c_k (r^2 - z_i)^k on the interval z_i < r^2 <= z_{i+1} (Andrea::eval,
       src/tabulate.h:188-207); for r^2 <= z_0, +inf if spline_hs, else the exact terms.        */
    const int* spline_begin;  /* n_types^2 + 1 offsets into spline_r2; >= 2 knots a pair    */
    const double* spline_r2;  /* the knots of every pair, ascending within a pair          */
    const double* spline_coef;/* 6 an interval; pair ab's start at 6 (spline_begin[ab] - ab) */
    const int* spline_hs;     /* n_types^2 KnotData::hardsphere_repulsion; NULL: none       */
    /* Hamiltonian::energy's `maxenergy` (src/energy.cpp:1189-1193, 1227-1241): each state's terms
       (self, Nonbonded, Ewald) are summed in order up to and including the first that is
       >= maxenergy or NaN.  maxenergy_set 0: +inf (every term summed).  Systems with it set
       run in the chain kernel (FP32C form, whatever their precision), also in batches.     */
    int maxenergy_set;
    double maxenergy;
    /* pipelined kernel, systems with a cell list: 0 = each move copies the occupied slots of its
       stencil cells only (the library's choice); 1 = whole cells; 2 = occupied slots when the
       system holds more particles than cells, else whole cells.  Batches that mix system shapes
       (a job server) run faster when most chains take the same code path.                   */
    int cell_staging;
} fau_sys_desc;

/* Per-term energies in kT (Hamiltonian term order: self, nonbonded, ewald). */
typedef struct fau_energy_terms {
    double self;        /* ParticleSelfEnergy                                   */
    double nonbonded;   /* Nonbonded pair sum                                   */
    double ewald_rec;   /* Ewald reciprocal energy                              */
    double ewald_surf;  /* Ewald surface energy                                 */
    double total;       /* sum as Hamiltonian::energy: ((self+nb)+ewald)        */
} fau_energy_terms;

/* Result of one trial move. */
typedef struct fau_trial_result {
    double du;          /* getEnergyChange(new, old) including the inf/NaN policy */
    double du_nonbonded;/* finite parts of the change, per term                   */
    double du_ewald;    /* reciprocal + surface                                   */
    double err_scale;   /* sum of |term| magnitudes the change was summed from    */
    int accepted;       /* Metropolis outcome (committed on the device if 1)      */
    int new_inf;        /* trial energy is +inf (hard-sphere overlap)             */
    int old_inf;        /* accepted-state energy is +inf                          */
    int pad;
} fau_trial_result;

/* One trial move proposal, produced on the host from the reference's RNG
 * stream (AtomicTranslateRotate::_move src/move.cpp:267-293,
 * TranslateRotate::_move src/move.cpp:1670-1689).                          */
enum fau_move_kind {
    FAU_MOVE_NONE = -1,      /* empty Change: only the Metropolis draw is consumed */
    FAU_MOVE_ATOMIC = 0,     /* translate particle `index` by dr                    */
    FAU_MOVE_MOLECULAR = 1,  /* translate group `index` by dr, then rotate by quat  */
    FAU_MOVE_VOLUME = 2      /* VolumeMove (src/move.cpp:994-1006): index = fau_volume_method,
                                dr[0] = (slump() - 0.5) dV; new volume exp(ln V + dr[0]);
                                single-system proposal streams only                 */
};
typedef struct fau_proposal {
    int32_t kind;       /* fau_move_kind                                           */
    int32_t index;      /* absolute particle index or group index                  */
    double dr[3];       /* displacement (angstrom)                                 */
    double quat[4];     /* rotation quaternion w,x,y,z (molecular only)            */
    double u;           /* Metropolis uniform in [0,1)                             */
} fau_proposal;

typedef struct fau_run_stats {
    int64_t moves;          /* moves performed                                    */
    int64_t accepted;       /* moves accepted                                     */
    int64_t pair_evals;     /* pair interactions evaluated (old + new)            */
    int64_t k_updates;      /* Ewald k-vector x moved-atom phase updates          */
    double energy_change;   /* sum of accepted dU (sum_of_energy_changes)         */
    double energy;          /* running total energy after the run                 */
    double max_rel_err;     /* the largest error of the FP32 energy changes against FP64
                               re-evaluations of audit probes (each launch ends with one
                               move evaluated on the final state, not decided), relative
                               to max(|dU|, S), since the system was made; 0 for the plain
                               FP64 form (fau_get_audit gives the other measures)     */
    double device_ms;       /* device time of the run (CUDA events)               */
} fau_run_stats;

/* Parameters of a batched run over many independent systems (replicas,
 * parallel-tempering walkers or served jobs).                               */
typedef struct fau_sampler fau_sampler; /* device analysis accumulators, see fau_sampler_create */

typedef struct fau_batch_params {
    int64_t moves;            /* moves per system in this launch (when moves_per_system is NULL) */
    const int64_t* moves_per_system; /* optional per-system move counts; under parallel tempering
                                 each walker's block length between swaps (e.g. 1,000 sweeps
                                 = 1000 N_i moves), replacing swap_interval_moves for it   */
    uint64_t seed;            /* counter-based RNG key                                    */
    uint64_t counter_base;    /* first move counter (continue a stream across launches)   */
    double dp;                /* translational displacement (angstrom)                    */
    double dprot;             /* rotational displacement (rad) for molecular systems      */
    int swap_interval_moves;  /* > 0: parallel-tempering swap after each block of this many
                                 moves per system (odd/even partners); 0: no swaps        */
    int n_swap_blocks;        /* number of swap blocks when swap_interval_moves > 0       */
    const double* temperatures; /* n temperatures (K) of the PT ladder, or NULL             */
    int threads;              /* CTA size: 96, 160, 288 -> the pipelined kernel with 2, 4, 8
                                 compute warps (molecular systems: the pipelined molecular
                                 kernel in 256-thread CTAs); 512 -> as 160, molecular
                                 systems in 512-thread CTAs (1 preparing + 15 compute warps);
                                 128, 256 -> the chain kernel for every system;
                                 0 -> chosen per launch: 8 compute warps when every pipelined
                                 chain fits on the GPU at once (two CTAs an SM) and no chain
                                 kernel or time budget shares the launch, else 4; molecular
                                 systems alone in a launch without a time budget in
                                 512-thread CTAs when every chain fits at once (one an SM),
                                 else 256.  The width sets the FP32 summation order: a fixed
                                 width keeps a system's chain independent of the rest of
                                 the batch                                              */
    const uint32_t* streams;  /* optional per-system RNG stream ids (default: batch index)  */
    const uint64_t* counters; /* optional per-system first move counter (default:
                                 counter_base); a system's moves depend only on its
                                 (seed, stream, counter), not on the rest of the batch   */
    const double* dp_per_system;    /* optional per-system dp (overrides dp)             */
    const double* dprot_per_system; /* optional per-system dprot (overrides dprot)       */
    uint64_t* cycles_out;     /* optional, n entries: SM clock cycles each system's chain
                                 took in this call (summed over swap blocks)             */
    fau_sampler* sampler;     /* optional device analysis sampled after every block, inside
                                 the launch's CUDA graph (no host round trip)             */
    const int* sample_slots;  /* optional n sampler slots (default: system i -> i mod n_slots) */
    int sample_interval_moves; /* with a sampler and no PT: blocks of this many moves per
                                 system; under PT the swap blocks are the sample blocks   */
    int n_sample_blocks;      /* number of sample blocks (no PT)                          */
    uint64_t time_budget_ns;  /* > 0 (no PT, no sampler): each system's chain ends at the first
                                 move boundary after this many ns of its own, or after its
                                 move count; a chain split this way continues exactly as one
                                 launch would (resume it at counter + moves done)        */
    int64_t* moves_out;       /* optional, n entries: moves (proposals) each system performed */
    /* parallel-tempering record (both optional, n_swap_blocks * n entries, round-major): the
       system holding each temperature slot after each round's swaps, and each system's running
       energy (kT of its own Hamiltonian) when the round's swaps were decided.  With the slot
       order of the round before (identity before the first), the temperatures and the
       counter-based uniforms, every swap decision can be recomputed by the caller.        */
    int* swap_slots_out;
    double* swap_energy_out;
    int no_audit;             /* 1: no audit probe (see fau_batch_stats.du_err_*)           */
    /* NPT in the batch (no PT, sampler or time budget; `moves` for every system): n_volume_blocks
       blocks of volume_interval_moves moves per system, each followed by one VolumeMove per
       system (src/move.cpp:994-1006): V' = exp(ln V + (u_a - 1/2) volume_dv), scaled by
       volume_method (fau_volume_method) and decided as fau_volume_move decides it on u_b.  u_a
       and u_b: Philox4x32-10 keyed by seed ^ 0x5DEECE66D on the counter (v mod 2^32, v / 2^32,
       stream, 9) for the system's volume move v = (counter + counter_base) / volume_interval_moves
       + block, as 53-bit uniforms from words (0, 1) and (2, 3); volume_dv = 0: no volume move */
    int volume_interval_moves;
    int n_volume_blocks;
    double volume_dv;
    int volume_method;
} fau_batch_params;

typedef struct fau_batch_stats {
    int64_t moves;
    int64_t accepted;
    int64_t pair_evals;
    int64_t k_updates;
    int64_t swaps_attempted;
    int64_t swaps_accepted;
    double device_ms;
    /* The error of the FP32 energy changes against FP64, for every launch: after its last move
     * each chain of the pipelined kernel evaluates one more (its next proposal, not decided or
     * committed) and an FP64 re-evaluation of the same move on the same state follows.  Largest
     * |dU32 - dU64| / max(|dU64|, S) (S: the sum of |summands|) and / |dU64| (|dU64| > 1e-3 kT)
     * over the batch's systems since they were made, and the probes of this call. */
    double du_err_scaled_max;
    double du_err_rel_max;
    int64_t du_err_samples;
    int64_t volume_attempted; /* volume moves of NPT blocks (also counted in moves/accepted) */
    int64_t volume_accepted;
} fau_batch_stats;

typedef struct fau_ctx fau_ctx;
typedef struct fau_sys fau_sys;

/* ---- library ------------------------------------------------------------- */
int fau_abi_version(void);
const char* fau_strerror(int status);
const char* fau_last_error(void);   /* detail of the last failure on this thread */

/* ---- context: one GPU, one stream, an HBM budget ------------------------- */
int fau_ctx_create(int device, size_t hbm_budget_bytes, fau_ctx** out);
int fau_ctx_destroy(fau_ctx* ctx);
int fau_ctx_hbm_used(const fau_ctx* ctx, size_t* used_bytes);

/* ---- systems ------------------------------------------------------------- */
/* Device bytes a system would hold (admission by HBM footprint). */
int fau_sys_footprint(const fau_sys_desc* desc, size_t* bytes);
/* Upload a Space + Hamiltonian; builds k-vectors (PolicyIonIon::updateBox,
 * src/energy.cpp:133-186), Q(k) (updateComplex, :191-206) and cell lists. */
int fau_sys_create(fau_ctx* ctx, const fau_sys_desc* desc, fau_sys** out);
int fau_sys_destroy(fau_sys* sys);
/* Deep device-to-device copy of a resident system in the same context (as the
 * reference builds a second State from one input, src/montecarlo.cpp:101-111):
 * replicas and jobs that share an initial state.  Counters start at zero. */
int fau_sys_clone(const fau_sys* src, fau_sys** out);
/* Checkpoint and resume: the exact device state of a system -- positions, fixed-point records,
 * mass centres, Q(k) with its FP32 pending sums, the cell lists in their slot order, the running
 * energy and its float-float part, the surface dipole, the temperature scale and the counters --
 * as an opaque blob of fau_sys_state_size bytes.  Loaded into a system made from the same
 * descriptor (with the saved box), the chains continue bit for bit as if never stopped: the
 * reference's state file (SaveState src/analysis.cpp:586-690, with its random-move and
 * random-global engines, src/faunus.cpp:430-470) carries positions only, whose rebuilt Q(k) and
 * cell order would change the last bits of later energy changes.  Device-RNG chains resume at
 * their next (seed, stream, counter); host streams from fau_movegen_get_state. */
int fau_sys_state_size(const fau_sys* sys, size_t* bytes);
int fau_sys_save_state(fau_sys* sys, void* buf, size_t bytes);
int fau_sys_load_state(fau_sys* sys, const void* buf, size_t bytes);
/* Number of Ewald k-vectors (0 without Ewald). */
int fau_sys_num_kvectors(const fau_sys* sys, int* k);

/* Full energy, Change::everything (Hamiltonian::energy src/energy.cpp:1227-1241),
 * evaluated on the device in FP64 from the resident state. */
int fau_energy_total(fau_sys* sys, fau_energy_terms* out);

/* One trial move, host-fed proposal and uniform: dU (trial minus accepted),
 * Metropolis on u01, commit on accept. Mirrors performMove for a single
 * transrot (src/move.cpp:267-293) or moltransrot (:1670-1689) move. */
int fau_trial_atomic(fau_sys* sys, int particle, const double dr[3], double u01,
                     fau_trial_result* out);
int fau_trial_group(fau_sys* sys, int group, const double dr[3], const double quat[4],
                    double u01, fau_trial_result* out);

/* Two-phase form of one trial move for an EnergyTerm-level integration, where
 * the caller's MetropolisMonteCarlo decides: fau_energy_change evaluates the
 * trial (Hamiltonian::updateState + energy of both states, src/energy.cpp:
 * 1227-1252) and keeps it pending on the device; fau_commit_pending(accept=1)
 * is State::sync trial -> accepted, accept=0 is accepted -> trial (the device
 * accepted state was never modified).  One pending move per system. */
int fau_energy_change(fau_sys* sys, const fau_proposal* proposal, fau_trial_result* out);
int fau_commit_pending(fau_sys* sys, int accept);

/* Run a stream of host-generated proposals back to back in one persistent
 * device kernel (one CTA per chain).  accepted_out (n bytes) and du_out
 * (n doubles) are optional host buffers. */
int fau_run_proposals(fau_sys* sys, const fau_proposal* proposals, int n,
                      uint8_t* accepted_out, double* du_out, fau_run_stats* stats);

/* Advance n independent systems with device-generated (Philox4x32-10)
 * proposals in one launch per swap block; PT swaps between blocks.
 * Parallel tempering (ParallelTempering::_move, src/move.cpp:883-923, with
 * OddEvenPartner::generate, src/mpicontroller.cpp:69-83): round r draws the
 * partner parity p from Philox4x32-10 keyed by (seed ^ 0x5DEECE66D) at counter
 * {r, r >> 32, 0xFFFFFFFF, 7} (p = word0 & 1); temperature slots s = p, p + 2, ...
 * pair with s + 1 and exchange when u <= exp(x), u the 53-bit uniform of the
 * words 0, 1 at counter {r, r >> 32, s, 8}, x = (1/T_s - 1/T_{s+1}) (E_a - E_b),
 * E the running energies in absolute units (kT_i T_i of each walker's own
 * Hamiltonian).  r = counter_base / swap_interval_moves + block.  Walkers run
 * in descending order of their block's cost (moves x particles), so that the
 * largest begin first, each on an SM of its own while SMs remain.
 * Systems made with FAU_PREC_FP64 run as FP64 replica chains (the plain FP64
 * form's pair sums, GroupCutoff, Ewald phases and Metropolis decision, all on
 * the device; single-atom and rigid-molecule moves; no finite maxenergy): a
 * batch holds FP64 systems only or none, else FAU_ERR_ARG. */
int fau_run_batch(fau_ctx* ctx, fau_sys* const* systems, int n, const fau_batch_params* params,
                  fau_batch_stats* stats);

/* Host-fed proposals for n systems in one launch (one CTA per system):
 * proposals[offsets[i] .. offsets[i+1]) belong to systems[i].  accepted_out
 * and du_out (optional) are indexed like proposals.  FP64 systems run as FP64
 * replica chains, as in fau_run_batch. */
int fau_run_proposals_batch(fau_ctx* ctx, fau_sys* const* systems, int n, const fau_proposal* proposals,
                            const int64_t* offsets, uint8_t* accepted_out, double* du_out,
                            fau_batch_stats* stats);

/* Measured FP32 FMA throughput of the device (roofline denominator). */
int fau_measure_fp32_peak(fau_ctx* ctx, double* tflops_out);

/* ---- nonbonded energy without device allocation ---------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * a host engine that owns all device memory through its own pool and does not
 * let a plugin allocate (cudaMalloc/cudaFree synchronise the device and
 * fragment the pool), or a latency-critical loop that must not stall on an
 * allocation.  The caller passes DEVICE pointers for every input and for the
 * output; nothing is allocated or freed, by this library or any library it
 * calls.  E = sum_{i<j} u(r_ij) over all particles as one atomic group (the
 * Nonbonded energy of Change::everything for a single atomic group), FP64,
 * written to *energy_out (device) asynchronously on `stream` (a cudaStream_t;
 * NULL = default stream).  type[i] must lie in [0, n_types).
 * Scratch: one file-scope device array of FAU_NOALLOC_MAX_PARTICLES doubles
 * (512 KiB) that every GPU loading this library holds until the process exits;
 * larger n_particles is rejected with FAU_ERR_ARG.  The first call on a device
 * (and the first after its context was made again, e.g. by cudaDeviceReset)
 * looks up the array's device address; make that call before any stream
 * capture.  All calls share the array: calls that overlap on the GPU race.
 * Positions need not be wrapped: separations are reduced by whole box lengths
 * before the minimum image.  coulomb_cutoff must be > 0 for the cut and ewald
 * forms; pair_cutoff <= 0 means no truncation (as in fau_sys_desc). */
#define FAU_NOALLOC_MAX_PARTICLES 65536
typedef struct fau_nonbonded_args {
    int n_particles;
    double box[3];
    const double* pos;        /* device, n*3 xyz                     */
    const double* charge;     /* device, n                           */
    const int* type;          /* device, n                           */
    int n_types;
    const double* sigma2;     /* device, n_types^2 (LJ/WCA)          */
    const double* eps4;       /* device, n_types^2 in kT (LJ/WCA)    */
    const double* hs_sigma2;  /* device, n_types^2 (HS) or NULL      */
    int pair_terms;           /* fau_pair_term bits                  */
    int coulomb_type;         /* fau_coulomb_type                    */
    double bjerrum_length, coulomb_cutoff, coulomb_alpha, pair_cutoff;
} fau_nonbonded_args;
int fau_nonbonded_energy_noalloc(const fau_nonbonded_args* args, double* energy_out, void* stream);

/* ---- volume move ----------------------------------------------------------
 * VolumeMove + Isobaric + Metropolis (src/move.cpp:994-1006, src/energy.cpp:884-901,
 * src/montecarlo.cpp:139-187): the box is scaled to `new_volume` as
 * Space::scaleVolume (src/space.cpp:249-301) -- atomic groups scale every position,
 * molecular groups are unwrapped about their mass centre, the mass centre scaled and
 * the atoms translated with it; boundary() in the new box -- the trial state's full
 * energy (Nonbonded, Ewald with the new box's k-vectors and a full Q(k) update,
 * self) is computed on the device in FP64, the descriptor's Isobaric term
 * P V - (N + 1) ln V, if present, is added to both states (N: particles of atomic
 * groups plus molecular groups), and the move is accepted on u01 <= exp(-dU).  On acceptance the system
 * holds the new state (its tables rebuilt for the new box); on rejection it is
 * unchanged.  The running energy excludes the Isobaric term. */
enum fau_volume_method {
    FAU_VOLUME_ISOTROPIC = 0, /* Cuboid::setVolume (src/geometry.cpp:57-90) */
    FAU_VOLUME_XY = 1,
    FAU_VOLUME_Z = 2,
    FAU_VOLUME_ISOCHORIC = 3
};
int fau_volume_move(fau_sys* sys, double new_volume, int method, double u01, fau_trial_result* out);

/* ---- device analysis ------------------------------------------------------
 * AtomRDF (src/analysis.cpp:1556-1600) and SystemEnergy (src/analysis.cpp:339-357)
 * sampled on the device into per-slot accumulators (one slot per replica, or one
 * slot pooling several).  AtomRDF: every pair of atoms of types a and b (i < j when
 * a == b), |vdist| under minimum image, bin floor(r / dr) as Equidistant2DTable
 * (src/aux/equidistant_table.h:32-39), plus the summed volume for PairFunction's
 * normalisation g(r) = N <V> / (4 pi r^2 dr sum N) (src/analysis.cpp:724-737).
 * SystemEnergy: sum and sum of squares of the running total energy.  Only cuboid
 * 3-d sampling (no slicedir / thickness). */
typedef struct fau_sampler_desc {
    int n_slots;        /* independent accumulators                                  */
    int rdf_type_a;     /* AtomRDF name1 / name2 as atom type ids                     */
    int rdf_type_b;
    double rdf_dr;      /* bin width (angstrom)                                       */
    int rdf_bins;       /* bins kept (<= FAU_SAMPLER_MAX_BINS); 0: no RDF; farther
                           pairs are counted in a last "beyond" column                */
    int energy;         /* 1: sample the running total energy                         */
} fau_sampler_desc;
#define FAU_SAMPLER_MAX_BINS 12000
int fau_sampler_create(fau_ctx* ctx, const fau_sampler_desc* desc, fau_sampler** out);
int fau_sampler_destroy(fau_sampler* s);
int fau_sampler_reset(fau_sampler* s);
/* Sample `n` systems of the sampler's context now (asynchronous on the context's
 * stream); slots: n slot ids, or NULL for system i -> slot i mod n_slots. */
int fau_sampler_sample(fau_sampler* s, fau_sys* const* systems, int n, const int* slots);
/* Copy the accumulators out (each pointer optional): rdf_hist n_slots*(rdf_bins+1)
 * counts (last column: beyond the bins), rdf_volume_sum / rdf_samples per slot,
 * energy_sum / energy_sum2 / energy_samples per slot. */
int fau_sampler_read(fau_sampler* s, uint64_t* rdf_hist, double* rdf_volume_sum, int64_t* rdf_samples,
                     double* energy_sum, double* energy_sum2, int64_t* energy_samples);

/* ---- state access -------------------------------------------------------- */
int fau_get_positions(fau_sys* sys, double* xyz_out);          /* n*3 FP64 */
int fau_get_mass_centers(fau_sys* sys, double* xyz_out);       /* n_groups*3 */
int fau_get_cells(fau_sys* sys, int* cell_out);                /* n cell index or -1 */
int fau_get_cell_grid(const fau_sys* sys, int dims_out[3]);
int fau_get_box(const fau_sys* sys, double box_out[3]);         /* cuboid side lengths */
int fau_get_running_energy(fau_sys* sys, double* energy_out);  /* FP64 running total */
/* Recompute the FP64 total energy and make it the running energy (after a start
 * from an infinite energy, where initial + sum of changes is not defined). */
int fau_refresh_energy(fau_sys* sys, double* energy_out);
/* Move counters since the system was created: {moves, accepted, pair
 * evaluations, k-vector updates} (Move::number_of_attempted_moves and
 * number_of_accepted_moves, src/move.h:50-59, summed over moves). */
int fau_get_counters(fau_sys* sys, int64_t counters_out[4]);
int fau_set_temperature_scale(fau_sys* sys, double scale);     /* beta multiplier (PT) */
/* Rebuild Q(k) in FP64 from the resident positions; returns the largest
 * |Q_cumulative - Q_rebuilt| before replacing (drift of the running Q). */
int fau_q_rebuild(fau_sys* sys, double* max_abs_drift_out);
int fau_get_q(fau_sys* sys, double* q_out);                    /* K complex as 2K doubles */
/* The resident Ewald k-vector table in its order (PolicyIonIon::updateBox, src/energy.cpp:133-186):
 * n_out 3K integer vectors n, k_out 3K wavevectors (2 pi)(n / L), ak_out K FP64 A_k; each optional. */
int fau_get_kvectors(fau_sys* sys, int* n_out, double* k_out, double* ak_out);
/* The system's audit since it was made (systems run in the pipelined kernel): err_out[0] the
 * largest |dU32 - dU64| / max(|dU64|, S), err_out[1] the largest / |dU64| (|dU64| > 1e-3 kT);
 * samples the probes evaluated. */
int fau_get_audit(fau_sys* sys, double err_out[2], int64_t* samples);

/* ---- host move generator (reference RNG stream) ---------------------------
 * std::mt19937 streams `slump` (Move::slump, src/move.cpp:21) and `random`
 * (global, src/random.cpp:62) drawn in the reference order; see
 * MoveCollection::sample (src/move.cpp:513-526),
 * AtomicTranslateRotate::_move (:267-293) and TranslateRotate::_move
 * (:1670-1689); randomUnitVector src/core.cpp:249-261. */
typedef struct fau_movegen fau_movegen;
typedef struct fau_move_desc {
    int kind;            /* FAU_MOVE_ATOMIC (transrot), FAU_MOVE_MOLECULAR (moltransrot) or
                            FAU_MOVE_VOLUME (volume)                                      */
    double repeat;       /* weight in the move collection (Move::repeat)                  */
    double dp;           /* translational displacement                                    */
    double dprot;        /* rotational displacement (rad)                                 */
    double dir[3];       /* translation directions                                        */
    int n_groups;        /* candidate groups (Space::findMolecules of the molecule)       */
    const int* groups;   /* group indices                                                 */
    const double* type_dp;    /* n_types AtomData::dp, NaN = unset (transrot); may be NULL */
    const double* type_dprot; /* n_types AtomData::dprot, NaN = unset; may be NULL         */
    int volume_method;   /* FAU_MOVE_VOLUME: fau_volume_method; dp is dV (VolumeMove::_from_json,
                            src/move.cpp:986-993), n_groups may be 0                    */
} fau_move_desc;
int fau_movegen_create(const fau_sys_desc* space, const fau_move_desc* moves, int n_moves,
                       uint32_t slump_seed, uint32_t random_seed, int default_seeds,
                       fau_movegen** out);
int fau_movegen_destroy(fau_movegen* gen);
/* Fill n proposals (one performMove each). */
int fau_movegen_generate(fau_movegen* gen, fau_proposal* out, int n);
/* Serialise / restore both engines (std::mt19937 text form, as Random::to_json). */
int fau_movegen_get_state(const fau_movegen* gen, char* buf, size_t buflen);
int fau_movegen_set_state(fau_movegen* gen, const char* state);

/* ---- splined pair potentials (host only) ----------------------------------
 * Tabulate::Andrea::generate (src/tabulate.h:212-298): quintic pieces in z = r^2 that match
 * f, f' and f'' (central differences, step 1e-4) at both ends, each as long as 11 checks keep
 * |spline - f| <= utol and, with ftol > 0, |spline' - f'| <= ftol; knots from zmax down to zmin,
 * at most 1200 intervals. Writes the knots (ascending) and 6 coefficients an interval; *n_knots
 * = intervals + 1; FAU_ERR_ARG when cap is too small or no interval meets the tolerance. */
typedef double (*fau_scalar_fn)(double z, void* ctx);
int fau_andrea_generate(fau_scalar_fn f, void* ctx, double zmin, double zmax, double utol, double ftol,
                        int cap, double* r2_out, double* coef_out, int* n_knots);

/* SplinedPotential::from_json + createKnots (src/potentials.cpp:1513-1597) for atom types a, b:
 * f = the sum of desc's pair terms (FAU_PAIR_SPLINE ignored) between two particles of those
 * types with charges charge_a, charge_b; rmin from `rmin_start` (0.5 (sigma_a + sigma_b)) moved
 * in steps of 0.01 until |f| is within [u_at_rmin / 1.1, 1.1 u_at_rmin] (findLowerDistance),
 * rmax from `rmax_start` (<= 0: 10 rmin_start) moved out until |f| <= u_at_rmax
 * (findUpperDistance); hardsphere_repulsion kept only where the spline at rmin^2 + 0.01 is >= 0. */
typedef struct fau_spline_opts {
    double utol;       /* default 1e-3 kT                                                   */
    double ftol;       /* default 1e-2; <= 0: no derivative check                          */
    double u_at_rmin;  /* default 20 kT                                                     */
    double u_at_rmax;  /* default 1e-6 kT                                                   */
    double rmax_start; /* "rmax" or the cutoff_g2g default; <= 0: 10 rmin_start             */
    int hardsphere;    /* "hardsphere": +inf below the first knot where repulsive           */
    int pad;
} fau_spline_opts;
int fau_spline_tabulate(const fau_sys_desc* desc, int type_a, int type_b, double charge_a, double charge_b,
                        double rmin_start, const fau_spline_opts* opts, int cap, double* r2_out,
                        double* coef_out, int* n_knots, int* hs_out);

#ifdef __cplusplus
}
#endif
#endif /* FAU_GPU_H */
