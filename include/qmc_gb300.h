/*
 * qmc_gb300.h -- C ABI of the GB300 (sm_103a) kernels behind the QMCTorch VMC
 * hot path: Slater-Jastrow wave function values, local energies and
 * Metropolis sampling.
 *
 * The reference (QMCTorch 0.4.0) is pure Python/PyTorch and has no native
 * interface; each entry point below replaces the reference Python function
 * cited beside it (paths relative to the QMCTorch repository). A binding
 * (ctypes, cffi, pybind11) passes plain device pointers and sizes:
 *
 *   - every pointer argument is a CUDA device pointer unless stated;
 *   - FP64 arrays are row-major and contiguous;
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy stream);
 *   - the caller owns every buffer, including the scratch workspace whose
 *     size the *_scratch_bytes functions report;
 *   - calls are asynchronous on `stream`; the return value reports argument
 *     and launch errors only (0 = QMC_OK).
 */
#ifndef QMC_GB300_H
#define QMC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum qmc_status {
  QMC_OK = 0,
  QMC_ERR_ARG = 1,         /* null pointer, negative size, bad mode */
  QMC_ERR_SHAPE = 2,       /* sizes beyond the compiled limits */
  QMC_ERR_SCRATCH = 3,     /* scratch buffer too small */
  QMC_ERR_LAUNCH = 4,      /* CUDA launch / runtime error */
  QMC_ERR_UNSUPPORTED = 5, /* option not implemented */
  QMC_ERR_STATIC_LIMIT = 6, /* batch needs more than QMC_STATIC_SCRATCH_BYTES (qmc_wf_psi_static) */
  QMC_ERR_TIMEOUT = 7       /* a bounded wait of a pipelined kernel ran out (qmc_mo_eval_tc_status) */
};

/* Compile-time limits of the kernels. */
#define QMC_MAX_NSPIN 64   /* electrons per spin channel */
#define QMC_MAX_COMP 6     /* AO components sharing one exponent set */

/* Determinant recipes (SlaterPooling, qmctorch/wavefunction/pooling/slater_pooling.py). */
#define QMC_DET_EXCITATION 0 /* ground state + single/double excitations via A^-1 B
                                (det_unique_single_double 147-260,
                                 operator_unique_single_double 437-636) */
#define QMC_DET_EXPLICIT 1   /* one LU per unique column set (det_explicit 96-111,
                                operator_explicit 348-409) */

/* Arithmetic of the fused kernels. QMC_PREC_FP64: the plain method, FP64
   throughout. QMC_PREC_MIXED: AO values and derivatives, the AO->MO
   contraction, the Jastrow factor and the Slater LU in FP32; positions and
   atom coordinates held as unevaluated FP32 pairs (hi + lo), so that
   electron-nucleus and electron-electron differences keep FP64-level
   accuracy in FP32 arithmetic; spin determinant products, psi, local-energy
   sums and one iterative-refinement step of the solves that feed the kinetic
   energy in FP64; CI sums as FP32 ratios to the ground-state determinant
   scaled by its FP64 value. The staged module kernels
   (qmc_ao_eval, qmc_mo_eval, qmc_jastrow_ee, qmc_slater) are FP64 always;
   qmc_mo_eval_tc is the mixed-precision (tensor-core) AO->MO module kernel. */
#define QMC_PREC_FP64 0
#define QMC_PREC_MIXED 1

/*
 * Wave-function description. Built once per molecule by the host layer from
 * the basis namespace (AtomicOrbitals.__init__, atomic_orbitals.py:16-102),
 * the CI configurations (OrbitalConfigurations.get_configs,
 * orbital_configurations.py:14-63; ExcitationMask, orbital_projector.py:97-189)
 * and the trainable parameters (ao.bas_exp, mo.mo_modifier,
 * jastrow.jastrow_kernel.weight, fc.weight), which the kernels read in place.
 *
 * AO "groups": consecutive AOs on one atom whose primitive exponents are
 * identical (cartesian components of a shell, general-contraction columns).
 * One exp() per (electron, group primitive) serves every AO of the group.
 */
typedef struct qmc_wf_desc {
  int32_t nelec, nup, ndown;
  int32_t natom;
  int32_t nao;       /* cartesian AOs */
  int32_t nmo;       /* columns of mo_scf / mo_modifier */
  int32_t nmo_used;  /* columns read by the determinants (highest occupied + 1) */
  int32_t ngroup;    /* AO groups */
  int32_t ngprim;    /* primitives over all groups */
  int32_t nweight;   /* AO-primitive weights (= basis entries) */
  int32_t contract;  /* 0 reproduces the uncontracted-basis value path (atomic_orbitals.py:246-249) */
  int32_t use_jastrow;
  int32_t precision; /* QMC_PREC_FP64 or QMC_PREC_MIXED (fused psi / local energy / Metropolis) */
  /* basis tables */
  const double* atom_coords;  /* [natom*3] */
  const double* atom_charge;  /* [natom] */
  const int32_t* group_atom;  /* [ngroup] */
  const int32_t* group_prim;  /* [ngroup+1] offsets into the group primitive arrays */
  const int32_t* group_ao;    /* [ngroup+1] AO ranges */
  const int32_t* gprim_entry; /* [ngprim] index of the exponent in bas_exp */
  const double* bas_exp;      /* [nentries] trainable exponents (ao.bas_exp) */
  const int32_t* ao_k;        /* [nao*3] cartesian powers kx, ky, kz */
  const int32_t* ao_wofs;     /* [nao] offset of the AO's weights (one per group primitive) */
  const int32_t* weight_entry;/* [nweight] basis entry (bas_exp index) of each AO weight; a group
                                 whose components' exponents differ is evaluated per component */
  const double* ao_wd;        /* [nweight] bas_coeffs * norm (derivative / contracted path) */
  const double* ao_wv;        /* [nweight] weights of the value path when contract == 0, else NULL */
  const double* mo_scf;       /* [nao*nmo] */
  const double* mo_modifier;  /* [nao*nmo] */
  /* Jastrow: Pade e-e kernel w0 r / (1 + w r), w0 = 0.25 same spin, 0.5 opposite */
  const double* jastrow_w;    /* [1] */
  /* CI expansion */
  int32_t det_mode;           /* QMC_DET_EXCITATION or QMC_DET_EXPLICIT */
  int32_t ncfg;
  int32_t max_orb[2];         /* excitation mode: highest orbital + 1 per spin */
  int32_t ndet[2];            /* unique spin determinants per spin */
  const int32_t* det_table[2];/* excitation: [ndet*5] (order, i0, i1, i2, i3) flat indices into
                                 A^-1 A_virt (n x (max_orb-n)); explicit: [ndet*n] column sets */
  const int32_t* cfg_det[2];  /* [ncfg] spin determinant of each configuration */
  const double* ci_weight;    /* [ncfg] (fc.weight) */
  double e_nuc;               /* nuclear repulsion (wf_base.py:97-116) */
  /* Electron-nucleus Pade Jastrow (optional): log J gains
     sum_{i,A} r_iA / (1 + w_en r_iA), the same static weight 1 for every pair
     (JastrowFactorElectronNuclei, jastrow_factor_electron_nuclei.py:9-161, with
     elec_nuclei/kernels/pade_jastrow_kernel.py:8-116). use_jastrow above selects
     the e-e factor and use_jastrow_en this one; with both, J is their product
     (CombineJastrow, combine_jastrow.py:7-195). */
  int32_t use_jastrow_en;
  const double* jastrow_en_w;     /* [1] (jastrow_kernel.weight of the e-n factor) */
  const double* jastrow_en_atoms; /* [natom*3] nucleus positions of the e-n factor */
  /* Radial part of the AOs (AtomicOrbitals.radial, radial_functions.py):
     QMC_RADIAL_GTO sums exp(-a r^2) (radial_gaussian_pure 241-320, the pyscf
     layout), QMC_RADIAL_STO is r^kr exp(-a r) (radial_slater 6-123, the ADF
     layout with cartesian harmonics), QMC_RADIAL_STO_PURE is exp(-a r)
     (radial_slater_pure 323-406). ao_kr: [nao] power of r of each AO (STO),
     may be NULL for GTO. */
  int32_t radial_type;
  const int32_t* ao_kr;
} qmc_wf_desc;

#define QMC_RADIAL_GTO 0
#define QMC_RADIAL_STO 1
#define QMC_RADIAL_STO_PURE 2

/* Scratch bytes for nwalkers walkers; kind 0 = psi, 1 = local energy. */
int64_t qmc_scratch_bytes(const qmc_wf_desc* d, int64_t nwalkers, int32_t kind);

/*
 * psi[w] = J(R_w) * sum_n c_n D_up,n D_down,n for positions pos[nwalkers][3*nelec].
 * Replaces SlaterJastrow.forward (slater_jastrow.py:243-286) and, squared,
 * WaveFunction.pdf (wf_base.py:241-247).
 */
int qmc_wf_psi(const qmc_wf_desc* d, const double* pos, int64_t nwalkers, double* psi,
               void* scratch, int64_t scratch_bytes, void* stream);

/*
 * qmc_wf_psi_static: psi[w] exactly as qmc_wf_psi computes it, for callers
 * that cannot allocate device memory on the call path -- for example a host
 * application that hands its whole HBM budget to its own pool allocator (a
 * cudaMalloc could fail or fragment that pool), a latency-critical loop in
 * which cudaMalloc/cudaFree would implicitly synchronize the device, or a
 * foreign-language binding that can pass device buffers but has no allocator
 * hook. It has no counterpart in the reference.
 *
 * The caller passes positions and the output; the workspace is a fixed
 * QMC_STATIC_SCRATCH_BYTES array compiled into this library (every GPU that
 * loads the library keeps it for the life of the process). Limit: batches
 * whose qmc_scratch_bytes(d, nwalkers, 0) exceeds QMC_STATIC_SCRATCH_BYTES are
 * rejected with QMC_ERR_STATIC_LIMIT and nothing is launched (about 174,000
 * walkers of H2O cc-pVDZ with single_double(4,4) in FP64: 96 bytes of
 * determinant values per walker). The library allocates
 * nothing: no cudaMalloc, cudaFree or allocating library call.
 *
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress, with that device current); make that first call
 * before any stream capture. All calls share the one array and it keeps the
 * previous call's contents; the kernel writes every element it reads, so
 * nothing needs clearing between calls, but calls that overlap on the GPU
 * (other streams, other host threads) race on it and must be serialized.
 */
#define QMC_STATIC_SCRATCH_BYTES (16 * 1024 * 1024)
int qmc_wf_psi_static(const qmc_wf_desc* d, const double* pos, int64_t nwalkers, double* psi,
                      void* stream);

/*
 * eloc[w] = -1/2 lap(psi)/psi + V_en + V_ee + V_nn; kinetic[w] and psi[w] are
 * optional (NULL to skip). Replaces WaveFunction.local_energy
 * (wf_base.py:184-215) with SlaterJastrow.kinetic_energy_jacobi
 * (slater_jastrow.py:312-344, get_kinetic_operator 449-482).
 */
int qmc_wf_local_energy(const qmc_wf_desc* d, const double* pos, int64_t nwalkers,
                        double* eloc, double* kinetic, double* psi,
                        void* scratch, int64_t scratch_bytes, void* stream);

/*
 * AO values. mode 0: ao[nw][ne][nao]; mode 1: gradient dao[nw][ne][nao][3];
 * mode 2: laplacian d2ao[nw][ne][nao]; mode 3: sum of the gradient components
 * ao[nw][ne][nao]; mode 4: all of ao, dao, d2ao.
 * Replaces AtomicOrbitals.forward (atomic_orbitals.py:131-218).
 */
int qmc_ao_eval(const qmc_wf_desc* d, const double* pos, int64_t nwalkers, int32_t mode,
                double* ao, double* dao, double* d2ao, void* stream);

/*
 * MO values mo[nrows][nmo] = ao[nrows][nao] @ (mo_scf * mo_modifier).
 * Replaces MolecularOrbitals.forward (molecular_orbitals.py:79-95).
 */
int qmc_mo_eval(const qmc_wf_desc* d, const double* ao, int64_t nrows, double* mo, void* stream);

/*
 * qmc_mo_eval_tc: the same product mo[nrows][nmo] = ao[nrows][nao] @ W on the
 * tensor cores (tcgen05.mma, FP32 accumulators in tensor memory), for the
 * mixed-precision method. Split-BF16 x3: each FP64 operand is split into
 * bf16 hi and lo parts and a_hi b_hi + a_hi b_lo + a_lo b_hi is accumulated
 * in FP32, so |mo - ao @ W| <= about 2e-5 * (|ao| @ |W|) elementwise (the FP64
 * qmc_mo_eval is exact to rounding). Replaces MolecularOrbitals.forward
 * (molecular_orbitals.py:79-95) when the wave function runs in mixed
 * precision. Limits: nmo <= 256 and shared memory (227 KB) for two
 * 128 x 2 nao' tiles of ao and one nmo' x 2 nao' tile of W in BF16 (nao', nmo'
 * rounded up to 16; nao <= 128 at nmo <= 128 fits), else QMC_ERR_SHAPE. If a
 * pipeline wait of the kernel runs out (1 s by default), the rows of the CTA
 * concerned are written as NaN and a device status word is set, which
 * qmc_mo_eval_tc_status reports.
 */
int qmc_mo_eval_tc(const qmc_wf_desc* d, const double* ao, int64_t nrows, double* mo,
                   void* stream);

/*
 * Status of the qmc_mo_eval_tc launches issued so far on the current device:
 * synchronizes `stream`, then returns QMC_ERR_TIMEOUT (and clears the status
 * word) if a pipeline wait of any of them ran out, else QMC_OK. No reference
 * counterpart (the reference has no asynchronous kernels).
 */
int qmc_mo_eval_tc_status(void* stream);

/*
 * Limit of each pipeline wait of qmc_mo_eval_tc, in nanoseconds, for launches
 * issued after the call (process-wide); returns the previous limit. Default
 * 1e9 (1 s). 0 makes every wait give up at once (the launch aborts: all rows
 * NaN, QMC_ERR_TIMEOUT), a test of the abort path that faults nothing. The
 * wait for the tensor core before tensor memory is released keeps 1 s. No
 * reference counterpart.
 */
uint64_t qmc_set_wait_limit_ns(uint64_t ns);

/*
 * Pade e-e Jastrow. jast[nw] (J), djast[nw][3][ne] (gradient, sum_grad = 0) or
 * [nw][ne] (sum_grad = 1), d2jast[nw][ne] (laplacian); NULL outputs are skipped.
 * Replaces JastrowFactorElectronElectron.forward
 * (jastrow_factor_electron_electron.py:124-260).
 */
int qmc_jastrow_ee(const qmc_wf_desc* d, const double* pos, int64_t nwalkers, double* jast,
                   double* djast, double* d2jast, int32_t sum_grad, void* stream);

/*
 * Electron-nucleus Pade Jastrow factor alone (use_jastrow_en must be set):
 * jast[nw] (J_en), djast[nw][3][ne] (sum_grad = 0) or [nw][ne] (sum_grad = 1),
 * d2jast[nw][ne] (laplacian); NULL outputs are skipped. Replaces
 * JastrowFactorElectronNuclei.forward (jastrow_factor_electron_nuclei.py:66-161).
 */
int qmc_jastrow_en(const qmc_wf_desc* d, const double* pos, int64_t nwalkers, double* jast,
                   double* djast, double* d2jast, int32_t sum_grad, void* stream);

/*
 * Slater determinants dets[nw][ncfg] from MO values mo[nw][ne][nmo_ld]
 * (SlaterPooling.forward, slater_pooling.py:64-80). If bop is not NULL, also
 * op[nw][ncfg] = Tr(A^-1 B) summed over spins for the operator matrix
 * bop[nw][ne][nmo_ld] (SlaterPooling.operator, slater_pooling.py:262-306).
 */
int qmc_slater(const qmc_wf_desc* d, const double* mo, const double* bop, int32_t nmo_ld,
               int64_t nwalkers, double* dets, double* op, void* scratch,
               int64_t scratch_bytes, void* stream);

/*
 * Coulomb terms per walker: v_en[nw] = -sum_e sum_A Z_A / r_eA and
 * v_ee[nw] = sum_{i<j} 1 / r_ij (either may be NULL). Replaces
 * WaveFunction.nuclear_potential / electronic_potential (wf_base.py:49-95).
 */
int qmc_potentials(const qmc_wf_desc* d, const double* pos, int64_t nwalkers, double* v_en,
                   double* v_ee, void* stream);

/* Scratch bytes for qmc_wf_psi_adjoint. */
int64_t qmc_adjoint_scratch_bytes(const qmc_wf_desc* d, int64_t nwalkers);

/*
 * Adjoint of psi (FP64, AO values recomputed, not stored): accumulates
 *   grad_exp[e]      += sum_w gout[w] d psi_w / d bas_exp[e]   (e < nentries)
 *   grad_W[a*ldw+j]  += sum_w gout[w] d psi_w / d W[a][j]      (j < nmo_used,
 *                       W = mo_scf * mo_modifier; d/d mo_modifier = this * mo_scf)
 *   grad_jastrow_w[0]+= sum_w gout[w] d psi_w / d w            (if use_jastrow)
 *   grad_jastrow_w[1]+= sum_w gout[w] d psi_w / d w_en         (if use_jastrow_en; the
 *                       array then holds two values)
 *   grad_ci[k]       += sum_w gout[w] d psi_w / d c_k
 * weight_entry[i] maps AO weight i (ao_wd index) to its basis entry. The outputs
 * are accumulated (zero them first); the summation order over walkers is not
 * fixed (atomic adds). Replaces the autograd backward of SlaterJastrow.forward
 * that Solver.evaluate_grad_manual runs with psi.backward(weight)
 * (solver.py:372-431).
 */
int qmc_wf_psi_adjoint(const qmc_wf_desc* d, const double* pos, int64_t nwalkers,
                       const double* gout, const int32_t* weight_entry, int32_t nentries,
                       double* grad_exp, double* grad_W, int32_t ldw, double* grad_jastrow_w,
                       double* grad_ci, void* scratch, int64_t scratch_bytes, void* stream);

/*
 * Electron-position gradients: grad[w][3*i + q] = d psi / d r_iq (pdf = 0) or
 * d psi^2 / d r_iq = 2 psi d psi / d r_iq (pdf != 0), by the Jacobi formula,
 * FP64. Replaces SlaterJastrow.gradients_jacobi (slater_jastrow.py:346-447),
 * used by WaveFunction.pdf(pos, return_grad=True) (wf_base.py:241-247).
 */
int64_t qmc_grad_scratch_bytes(const qmc_wf_desc* d, int64_t nwalkers);
int qmc_wf_gradients(const qmc_wf_desc* d, const double* pos, int64_t nwalkers, int32_t pdf,
                     double* grad, void* scratch, int64_t scratch_bytes, void* stream);

/* Scratch bytes for qmc_wf_local_energy_adjoint. */
int64_t qmc_eloc_adjoint_scratch_bytes(const qmc_wf_desc* d, int64_t nwalkers);

/*
 * Adjoint of the local energy (FP64, AO values and derivatives recomputed):
 * accumulates sum_w gout[w] d E_L(w) / d theta into the same outputs as
 * qmc_wf_psi_adjoint (grad_exp per basis entry, grad_W for
 * W = mo_scf * mo_modifier, grad_jastrow_w, grad_ci). The positions are held
 * fixed. Replaces the autograd backward of WaveFunction.local_energy
 * (wf_base.py:184-215 with kinetic_energy_jacobi, slater_jastrow.py:312-344)
 * that Solver.evaluate_grad_auto runs with loss.backward() (solver.py:352-370).
 */
int qmc_wf_local_energy_adjoint(const qmc_wf_desc* d, const double* pos, int64_t nwalkers,
                                const double* gout, const int32_t* weight_entry,
                                int32_t nentries, double* grad_exp, double* grad_W, int32_t ldw,
                                double* grad_jastrow_w, double* grad_ci, void* scratch,
                                int64_t scratch_bytes, void* stream);

/* Metropolis move types (Metropolis.configure_move, metropolis.py:179-225). */
#define QMC_MOVE_ALL_ELEC 0
#define QMC_MOVE_ONE_ELEC 1
#define QMC_MOVE_ALL_ELEC_ITER 2
#define QMC_PROBA_NORMAL 0
#define QMC_PROBA_UNIFORM 1

typedef struct qmc_metropolis_args {
  double* pos;            /* [nw][3*ne] walker positions, updated in place */
  int64_t nwalkers;
  int32_t nstep;
  int32_t ntherm;         /* >= 0 (the caller resolves negative values) */
  int32_t ndecor;
  int32_t move_type;      /* QMC_MOVE_* */
  int32_t proba;          /* QMC_PROBA_* */
  double step_size;
  uint64_t seed;          /* Philox key */
  uint64_t step_offset;   /* Philox counter offset (continue a chain) */
  double* samples;        /* [nsnap][nw][3*ne] kept positions, or NULL */
  int64_t nsnap;          /* capacity of samples in snapshots */
  int32_t* accepted;      /* [nw] accepted moves, accumulated, or NULL */
  double* psi_out;        /* [nw] psi at the final positions, or NULL */
  /* Replay inputs (tests): when not NULL they replace the generator.
     all-elec: proposals [nstep][nw][3*ne], uniforms [nstep][nw];
     single-electron: proposals [nstep][nmove][nw][3], uniforms [nstep][nmove][nw],
     electron_index [nstep][nw] (one-elec). */
  const double* proposals;
  const double* uniforms;
  const int32_t* electron_index;
} qmc_metropolis_args;

/* Scratch bytes for qmc_metropolis_run: the determinant work arrays and room
   for the walkers' current positions (launch plans that keep them out of
   shared memory). */
int64_t qmc_metropolis_scratch_bytes(const qmc_wf_desc* d, int64_t nwalkers);

/*
 * Launch plan of the all-electron Metropolis kernel for nwalkers walkers
 * (diagnostics, no counterpart in the reference): plan[0] walkers per block,
 * plan[1] threads per walker, plan[2] threads per block, plan[3] 1 when the
 * current positions live in the scratch instead of shared memory (no plan
 * with them in shared memory runs in one wave), plan[4] dynamic shared
 * memory bytes per block. Needs a CUDA device (occupancy query).
 */
int qmc_metropolis_plan(const qmc_wf_desc* d, int64_t nwalkers, int32_t* plan);

/*
 * Run nstep Metropolis steps for every walker in one persistent launch.
 * Replaces Metropolis.__call__ (metropolis.py:85-177) with move / _move /
 * _accept (227-298): Gaussian proposals of covariance sigma*I with
 * sigma = step_size / (2 sqrt(2 ln 2)) (quirk kept: per-coordinate standard
 * deviation sqrt(sigma)) or uniform proposals step*(2u-1); accept when
 * min(1, psi'^2/psi^2) - u >= 0, zero densities replaced by 1e-16.
 */
int qmc_metropolis_run(const qmc_wf_desc* d, const qmc_metropolis_args* a,
                       void* scratch, int64_t scratch_bytes, void* stream);

/*
 * qmc_metropolis_run for up to QMC_MAX_BATCH independent jobs in one launch
 * (no reference counterpart: the serving loop's continuous batching). Job j
 * is (descs[j], args[j]) with its own scratch[j] of scratch_bytes[j] bytes;
 * each job's walkers evolve exactly as in a qmc_metropolis_run call with the
 * same arguments (bitwise), whatever the other jobs are. Jobs may differ in
 * molecule, electron count, basis and CI expansion; they must share the
 * precision and the MO column class of the determinants (nmo_used <= 8,
 * 9..16 or 17..24); otherwise QMC_ERR_SHAPE. Each job runs the launch plan it
 * would get alone; the block size and shared memory are the largest over the
 * jobs. All-electron moves without replay inputs or psi_out only
 * (QMC_ERR_UNSUPPORTED).
 */
#define QMC_MAX_BATCH 32
int qmc_metropolis_run_batch(const qmc_wf_desc* descs, const qmc_metropolis_args* args,
                             void* const* scratch, const int64_t* scratch_bytes, int32_t njobs,
                             void* stream);

/* Arguments of qmc_drift_run (the drift-diffusion sampler). */
typedef struct qmc_drift_args {
  double* pos;            /* [nw][3*ne] in: start positions; out: final positions */
  int64_t nwalkers;
  int32_t nstep;
  int32_t ntherm;         /* >= 0 (the caller resolves negative values) */
  int32_t ndecor;
  double step_size;
  uint64_t seed;          /* Philox key */
  uint64_t step_offset;   /* Philox counter offset (continue a chain) */
  double* samples;        /* [nsnap][nw][3*ne] kept positions, or NULL */
  int64_t nsnap;          /* capacity of samples in snapshots */
  int32_t* accepted;      /* [nw] accepted moves, accumulated, or NULL */
  /* Replay inputs: all three or none. When given they replace the generator:
     electron_index [nstep][nw] (in [0, ne)), normals [nstep][nw][3] (the
     proposal noise, covariance sqrt(step_size) I already applied),
     uniforms [nstep][nw]. */
  const int32_t* electron_index;
  const double* normals;
  const double* uniforms;
} qmc_drift_args;

/* Scratch bytes for qmc_drift_run. */
int64_t qmc_drift_scratch_bytes(const qmc_wf_desc* d, int64_t nwalkers);

/*
 * Run nstep drift-diffusion Metropolis steps for every walker in one launch,
 * FP64. Replaces GeneralizedMetropolis.__call__ with move / _move / trans /
 * get_drift / _accept (generalized_metropolis.py:46-219) for the density psi^2
 * of the described wave function: each step moves one electron e (uniform)
 * of the call's START positions by step * drift_i(e) + eta, eta ~ N(0,
 * sqrt(step) I), drift = grad psi / psi (Jacobi formula); accepts when
 * min(1, T_if rho_f / (T_fi rho_i)) - u >= 0 with
 * T(x -> y) = exp(-|y - x - step drift(x)| / (2 step)) (the norm of the whole
 * walker vector), zero densities replaced by 1e-16. Samples are kept after
 * ntherm steps every ndecor steps; pos receives the final positions.
 */
int qmc_drift_run(const qmc_wf_desc* d, const qmc_drift_args* a, void* scratch,
                  int64_t scratch_bytes, void* stream);

/* Arguments of qmc_hmc_run (Hamiltonian Monte Carlo). */
typedef struct qmc_hmc_args {
  double* pos;            /* [nw][3*ne] in: start positions; out: final positions */
  int64_t nwalkers;
  int32_t nstep;
  int32_t ntherm;         /* >= 0 (the caller resolves negative values) */
  int32_t ndecor;
  int32_t traj_length;    /* leapfrog steps per trajectory (L >= 1) */
  double step_size;       /* leapfrog step eps */
  uint64_t seed;          /* Philox key */
  uint64_t step_offset;   /* Philox counter offset (continue a chain) */
  double* samples;        /* [nsnap][nw][3*ne] kept positions, or NULL */
  int64_t nsnap;          /* capacity of samples in snapshots */
  int32_t* accepted;      /* [nw] accepted trajectories, accumulated, or NULL */
  /* Replay inputs: both or none. momenta [nstep][nw][3*ne] (standard normal),
     uniforms [nstep][nw]. */
  const double* momenta;
  const double* uniforms;
} qmc_hmc_args;

/* Scratch bytes for qmc_hmc_run. */
int64_t qmc_hmc_scratch_bytes(const qmc_wf_desc* d, int64_t nwalkers);

/*
 * Run nstep Hamiltonian Monte Carlo steps for every walker in one launch,
 * FP64. Replaces Hamiltonian.__call__ with _step (hamiltonian.py:75-201) for
 * the density psi^2 of the described wave function: momenta p ~ N(0, I),
 * H = -log psi^2 + |p|^2 / 2, a leapfrog trajectory of traj_length steps of
 * size step_size with the force 2 grad psi / psi (Jacobi formula), the end
 * point rejected when exp(H_start - H_end) < u. Samples are kept after ntherm
 * steps every ndecor steps; pos receives the final positions.
 */
int qmc_hmc_run(const qmc_wf_desc* d, const qmc_hmc_args* a, void* scratch,
                int64_t scratch_bytes, void* stream);

/*
 * Compensated statistics of x[0..n) (local energies): stats[0] = mean,
 * stats[1] = unbiased variance, stats[2] = sqrt(stats[1] / n). Replaces the
 * torch.mean / torch.var / WaveFunction.sampling_error of
 * SolverBase.single_point (solver_base.py:316-387, wf_base.py:225-229).
 * Two passes of Neumaier-compensated sums merged in a fixed order: the result
 * depends on n only. stats is a device pointer.
 */
int64_t qmc_reduce_scratch_bytes(int64_t n);
int qmc_reduce_stats(const double* x, int64_t n, double* stats, void* scratch,
                     int64_t scratch_bytes, void* stream);

/*
 * Restricted Hartree-Fock integrals (host code, host pointers). The reference
 * takes its molecular orbitals from pyscf (RHF, qmctorch/scf/calculator/
 * pyscf.py:88-103); these replace pyscf's integrals over the basis functions
 * exactly as the AO layer evaluates them:
 *   chi_mu(r) = sum_{p : prim_ao[p] = mu} prim_coef[p] x^kx y^ky z^kz exp(-prim_exp[p] |r - C_p|^2)
 * (x, y, z relative to the centre C_p, cartesian powers prim_k[p*3..], total
 * degree <= 2). McMurchie-Davidson recursions, Boys function from its series.
 */
typedef struct qmc_gto_basis {
  int32_t nao;               /* contracted functions */
  int32_t nprim;             /* primitive entries */
  const int32_t* prim_ao;    /* [nprim] function of each entry */
  const double* prim_center; /* [nprim*3] */
  const double* prim_exp;    /* [nprim] */
  const double* prim_coef;   /* [nprim] contraction coefficient x primitive norm */
  const int32_t* prim_k;     /* [nprim*3] cartesian powers */
} qmc_gto_basis;

/* Overlap S, kinetic energy T and nuclear attraction V (-sum_C Z_C / |r - C|),
   each [nao*nao], of the basis over natom point charges. */
int qmc_scf_one_electron(const qmc_gto_basis* b, int32_t natom, const double* atom_xyz,
                         const double* atom_z, double* S, double* T, double* V);

/* Electron repulsion integrals (mu nu | la si) = eri[((mu*n + nu)*n + la)*n + si]
   (chemists' notation, all nao^4 entries, 8-fold symmetry filled; quartets whose
   Schwarz bound is below 1e-14 are 0). Threads: all host cores. */
int qmc_scf_eri(const qmc_gto_basis* b, double* eri);

/* Human-readable status. */
const char* qmc_status_string(int status);

/* Library version string. */
const char* qmc_version(void);

#ifdef __cplusplus
}
#endif

#endif /* QMC_GB300_H */
