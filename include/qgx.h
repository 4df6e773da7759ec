/*
 * qgx.h -- C ABI of the GB300 (sm_103a) VMC inner loop: Metropolis sampling, local
 * energies, per-sample log-derivatives, Gram matrices and the FP64 SR / MinSR solve.
 *
 * Conventions for every entry point:
 *   - all array arguments are DEVICE pointers owned by the caller (no allocation inside
 *     the library, apart from one lazily created cuSOLVER handle per device);
 *   - work is enqueued on the given stream and the call returns without synchronising;
 *   - the return value is a status code (QGX_OK on success); a non-zero status means
 *     nothing was enqueued (argument errors) or the launch failed (QGX_ERR_CUDA);
 *   - spin configurations are bit-packed: chain c occupies words
 *     spins[c*nw .. c*nw+nw-1], nw = (n+31)/32, bit (j%32) of word j/32 is 1 when
 *     site j holds +1 (spin up) and 0 when it holds -1;
 *   - random draws come from Philox4x32-10 keyed by the 64-bit seed; draw t of chain c
 *     uses counter (c, t & 0xffffffff, t >> 32, tag << 24).
 *
 * The reference interfaces each entry point replaces are cited as
 * path:line inside the reference project (ChenAo-Phys/quantax).
 */
#ifndef QGX_H_
#define QGX_H_

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* qgx_stream_t; /* == cudaStream_t */

#define QGX_OK 0
#define QGX_ERR_ARG 1          /* invalid argument (size, null pointer, layout) */
#define QGX_ERR_CUDA 2         /* a CUDA launch or runtime call failed */
#define QGX_ERR_TIMEOUT 3      /* a bounded device wait expired */
#define QGX_ERR_NONFINITE 4    /* non-finite value detected */
#define QGX_ERR_UNSUPPORTED 5  /* configuration outside the compiled kernels */
#define QGX_ERR_SOLVER 6       /* cuSOLVER returned an error */

#define QGX_PROPOSAL_LOCAL_FLIP 0    /* quantax.sampler.LocalFlip */
#define QGX_PROPOSAL_SPIN_EXCHANGE 1 /* quantax.sampler.SpinExchange */

/* diagonal-shifted Cholesky (minnorm_shift_eig): this library's FP64 factorisation (FP64
 * diagonal blocks and triangular solves, every trailing update an exact BF16-digit product on
 * the tensor cores; see qgx_cholesky) */
#define QGX_SOLVE_SHIFT 0
#define QGX_SOLVE_PINV 1   /* soft pseudo-inverse via eigh (minnorm_pinv_eig) */
/* diagonal-shifted system solved by FP64 conjugate gradients preconditioned with the FP32
 * Cholesky factor of the shifted matrix (cuSOLVER, BF16x9-emulated FP32); when that factor
 * breaks down it is recomputed once with 4 sqrt(n) 2^-24 tr(T) more on the diagonal.
 * info = -1 when the true FP64 residual stays above 1e-10 relative after 100 iterations
 * (the caller then falls back to QGX_SOLVE_SHIFT) */
#define QGX_SOLVE_SHIFT_MIXED 2
/* as QGX_SOLVE_SHIFT with cuSOLVER's FP64 Xpotrf (FP64 pipe) as the factorisation */
#define QGX_SOLVE_SHIFT_LIB 3

#define QGX_GRAM_FP32 0    /* FP32 SIMT FMA, FP32 accumulation */
#define QGX_GRAM_TF32 1    /* tcgen05 kind::tf32, FP32 accumulation in TMEM */
#define QGX_GRAM_BF16 2    /* tcgen05 kind::f16 with bf16 operands, FP32 accumulation */
#define QGX_GRAM_3XTF32 3  /* tcgen05 split-TF32 (hi*hi + hi*lo + lo*hi), FP32 accuracy */
#define QGX_GRAM_FP64 4    /* SIMT, exact FP32 products summed as float pairs: the Gram of the
                            * FP32 operand to about 48 bits (for solves that keep eigenvalues
                            * below FP32 resolution, e.g. lstsq_pinv_eig(rtol=1e-9)) */

/* ---- library ----------------------------------------------------------------- */
int qgx_abi_version(void);
const char* qgx_status_string(int status);
/* Human-readable text of the last error recorded by this thread ("" if none): a CUDA error,
 * or the reason an entry point rejected its arguments where it gives one. */
const char* qgx_last_error(void);
/* Empty this thread's qgx_last_error() text (a caller clears it before a call so that the
 * text it reads afterwards belongs to that call). Status plumbing of this library; no
 * counterpart in the reference, whose errors are Python exceptions. */
void qgx_clear_last_error(void);

/* ---- random numbers ------------------------------------------------------------ */
/* Raw Philox4x32-10 on n counters: out[4i..4i+3] = philox(ctr[4i..4i+3], key[0..1]).
 * Known-answer check of the generator shared by every sampler. Replaces the threefry
 * key handling of quantax/global_defs.py:54-91. */
int qgx_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out, int64_t n,
                      qgx_stream_t stream);

/* ---- configurations (quantax/utils/basis.py:121-219) ----------------------------- */
/* Uniform +-1 configurations (_rand_states, basis.py:121-125). */
int qgx_spins_init_uniform(uint32_t* spins, int64_t ns, int32_t n, uint64_t seed,
                           qgx_stream_t stream);
/* Exactly nup up spins per chain, independent uniform permutations
 * (_rand_Nconserved, basis.py:128-133). */
int qgx_spins_init_fixed_up(uint32_t* spins, int64_t ns, int32_t n, int32_t nup,
                            uint64_t seed, qgx_stream_t stream);
/* int8 +-1 <-> packed adapters for API parity with the reference's int8 spins. */
int qgx_spins_unpack(const uint32_t* spins, int8_t* out, int64_t ns, int32_t n,
                     qgx_stream_t stream);
int qgx_spins_pack(const int8_t* in, uint32_t* spins, int64_t ns, int32_t n,
                   qgx_stream_t stream);

/* ---- local operators -------------------------------------------------------------- */
/* A spin Hamiltonian compiled from a QuSpin-format op list
 * (quantax/operator/operator.py:187-238, 30-119) into device tables:
 *   diagonal:  c0 + sum_z Jz[k] s[iz[k]] + sum_zz Jzz[k] s[i] s[j]
 *   one-site flips: element f1_J[2k + (s_i>0)] for flipping site f1_i[k]
 *   two-site flips: element f2_J[4k + 2(s_i>0) + (s_j>0)] for flipping f2_ij[2k], f2_ij[2k+1]
 * A zero element means "no connection" (the reference's NaN / isclose(0) compaction,
 * operator.py:144-165). All pointers are device pointers. */
typedef struct {
  double c0;
  int32_t n_z;
  const int32_t* z_i;
  const double* z_J;
  int32_t n_zz;
  const int32_t* zz_ij; /* 2*n_zz */
  const double* zz_J;
  int32_t n_f1;
  const int32_t* f1_i;
  const double* f1_J; /* 2*n_f1 */
  int32_t n_f2;
  const int32_t* f2_ij; /* 2*n_f2 */
  const double* f2_J;   /* 4*n_f2 */
} qgx_operator_t;

/* Diagonal part only, per configuration (Operator.apply_diag, operator.py:83-93). */
int qgx_operator_diag(const qgx_operator_t* op, const uint32_t* spins, int64_t ns, int32_t n,
                      double* out, qgx_stream_t stream);

/* ---- RBM_Dense (quantax/model/shallow_nets.py:35-126) ------------------------------- */
/* Supported: n <= 1024 sites, m <= 1024 hidden units (padded internally to 128, 256, 384,
 * 512 or 1024 with zero weights). */
/* Number of floats of the per-parameter-set table used by every RBM kernel. */
int64_t qgx_rbm_table_floats(int32_t n, int32_t m);
/* Build the table from W (m x n row-major, eqx Linear layout), b (m) and the optional
 * visible bias a (n, may be NULL). Must be re-run after every parameter update. */
int qgx_rbm_prepare(const float* W, const float* b, const float* a, int32_t n, int32_t m,
                    float* table, qgx_stream_t stream);
/* log|psi(s)| = sum_i log cosh(W s + b)_i (+ a.s)   (Variational.__call__,
 * quantax/state/variational.py:325-347). */
int qgx_rbm_log_psi(const float* table, int32_t n, int32_t m, const uint32_t* spins,
                    int64_t ns, float* log_psi, qgx_stream_t stream);
/* nsteps Metropolis proposals on every chain, one warp per chain, theta resident
 * (Metropolis._partial_sweep/_single_sweep/_update, quantax/sampler/metropolis.py:246-322;
 * LocalFlip.propose common_samplers.py:28-33; SpinExchange common_samplers.py:58-162).
 * Draw t of chain c is step0 + t. spins are updated in place; log_psi receives
 * log|psi| of the final configurations; accepts (may be NULL) receives per-chain accept
 * counts. nbr (n x z int32, -1 padded) and hop are used by SPIN_EXCHANGE only. */
int qgx_rbm_sweep(const float* table, int32_t n, int32_t m, uint32_t* spins, float* log_psi,
                  int32_t* accepts, int64_t ns, int32_t nsteps, uint64_t seed, uint64_t step0,
                  float reweight, int32_t proposal, const int32_t* nbr, int32_t z, int32_t hop,
                  qgx_stream_t stream);
/* Local energies E_loc(s) = sum_s' H_ss' psi(s')/psi(s) with connected configurations
 * generated in-kernel (Operator.Oloc, quantax/operator/operator.py:510-562). */
int qgx_rbm_eloc(const float* table, int32_t n, int32_t m, const qgx_operator_t* op,
                 const uint32_t* spins, int64_t ns, double* eloc, qgx_stream_t stream);

/* ---- batched RBM sweeps and local energies ---------------------------------------- */
/* The serving loop's RBM jobs of one step in few launches: every job of one class (hidden-unit
 * width class, whether its table fits shared memory, proposal kind) runs in one launch, with
 * the job table passed as a kernel parameter. Each job's results (spins, log psi, accepts;
 * local energies) are bit-identical to its own qgx_rbm_sweep / qgx_rbm_eloc call. At most
 * QGX_RBM_BATCH_MAX_JOBS jobs per call; the structs and the operators they point to are read on
 * the host during the call only. */
#define QGX_RBM_BATCH_MAX_JOBS 64
typedef struct {
  const float* table; /* qgx_rbm_prepare's table */
  int32_t n, m;
  uint32_t* spins;    /* ns packed configurations, in / out */
  float* log_psi;     /* ns, out */
  int32_t* accepts;   /* ns accept counts, out (may be NULL) */
  int64_t ns;
  int32_t nsteps;
  int32_t proposal;   /* QGX_PROPOSAL_* */
  uint64_t seed, step0;
  float reweight;
  const int32_t* nbr; /* SpinExchange neighbour table (NULL for LocalFlip) */
  int32_t z, hop;
} qgx_rbm_sweep_job_t;
/* launches (may be NULL): the number of kernel launches made */
int qgx_rbm_sweep_batched(const qgx_rbm_sweep_job_t* jobs, int32_t njobs, int32_t* launches,
                          qgx_stream_t stream);
typedef struct {
  const float* table;
  int32_t n, m;
  const qgx_operator_t* op; /* host struct of device tables */
  const uint32_t* spins;
  int64_t ns;
  double* eloc;             /* ns, out */
} qgx_rbm_eloc_job_t;
int qgx_rbm_eloc_batched(const qgx_rbm_eloc_job_t* jobs, int32_t njobs, int32_t* launches, qgx_stream_t stream);
/* Per-sample log-derivatives O (ns x np, row stride ldo floats), np = m*n + m (+ n with
 * the visible bias), parameter order W (row-major), b, a (Variational.jacobian,
 * quantax/state/variational.py:424-511). */
int qgx_rbm_jacobian(const float* table, int32_t n, int32_t m, int32_t has_vbias,
                     const uint32_t* spins, int64_t ns, float* O, int64_t ldo,
                     qgx_stream_t stream);
/* Workspace bytes of qgx_rbm_obar. */
int64_t qgx_rbm_obar_workspace_bytes(int32_t n, int32_t m, int64_t ns);
/* Centred, scaled log-derivatives Obar = (O - mean_s O) * sqrt(r_s / ns) written in one
 * pass, and the weighted mean Omean = mean_s(O r) (np doubles)
 * (QNGD.get_Obar/_Omat_to_Obar, quantax/optimizer/sr.py:76-88). r may be NULL (all 1). */
int qgx_rbm_obar(const float* table, int32_t n, int32_t m, int32_t has_vbias,
                 const uint32_t* spins, const double* r, int64_t ns, float* Obar, int64_t ldo,
                 double* omean, void* workspace, int64_t workspace_bytes, qgx_stream_t stream);

/* qgx_rbm_obar for callers that cannot allocate device memory. No counterpart in the
 * reference. Some callers are not allowed to call cudaMalloc at all: a JAX/XLA FFI
 * custom-call handler runs inside the framework's executor, whose device memory belongs
 * to the framework's allocator, and a serving loop that reserved its HBM budget at start-up
 * must not allocate while jobs are running. This entry point takes the same inputs and
 * outputs as qgx_rbm_obar but keeps its scratch (tanh buffer, column partial sums, column
 * means) in one static device array of QGX_RBM_OBAR_STATIC_SCRATCH_BYTES bytes inside
 * the library; every GPU that loads the library holds that array until the process exits.
 * Requests needing more scratch (qgx_rbm_obar_workspace_bytes(n, m, ns) larger than the
 * array) return QGX_ERR_ARG and nothing is enqueued; qgx_last_error() then says why.
 * The first call on a device looks up the array's device address (cudaGetSymbolAddress)
 * with that device current; make that first call before any stream capture. The address is
 * cached per device with the CUDA context it belongs to; when the device's current context
 * changes (the primary context released and created again, e.g. by cudaDeviceReset) the next
 * call looks it up again, so that call too should come before any capture. All calls
 * share the array and it keeps the last call's contents (every region is fully written
 * before it is read, so nothing needs clearing): calls that overlap on the GPU, on
 * different streams of one device, race on it and must be serialised by the caller. */
#define QGX_RBM_OBAR_STATIC_SCRATCH_BYTES (32LL << 20)
int qgx_rbm_obar_noalloc(const float* table, int32_t n, int32_t m, int32_t has_vbias,
                         const uint32_t* spins, const double* r, int64_t ns, float* Obar,
                         int64_t ldo, double* omean, qgx_stream_t stream);

/* ---- RBM_Conv (quantax/model/shallow_nets.py:129-190) ---------------------------------
 * psi = prod_{c,x} cosh(theta_{c,x}), theta_{c,x} = b_c + sum_k W_c[(k - x + lo) mod L] s_k on an
 * L0 x L1 periodic lattice (L1 = 1 for a chain; lo = (L - 1) / 2 per axis, the circular SAME
 * convolution with a lattice-sized kernel). Parameters: W (channels x L0 x L1, row-major), then
 * b (channels). It is the dense RBM with n = L0 L1 visible and m = channels L0 L1 <= 2048
 * hidden units: qgx_rbm_log_psi / qgx_rbm_sweep / qgx_rbm_eloc run on its table with those
 * n and m. */
int64_t qgx_rbm_conv_table_floats(int32_t L0, int32_t L1, int32_t channels);
int qgx_rbm_conv_prepare(const float* params, int32_t L0, int32_t L1, int32_t channels, float* table,
                         qgx_stream_t stream);
/* Per-sample log-derivatives of the shared weights and biases (ns x (channels L0 L1 +
 * channels), row stride ldo floats, the parameter order above). */
int qgx_rbm_conv_jacobian(const float* table, int32_t L0, int32_t L1, int32_t channels,
                          const uint32_t* spins, int64_t ns, float* O, int64_t ldo, qgx_stream_t stream);

/* ---- ResConv (quantax/model/conv_nets.py:26-183) ----------------------------------- */
/* Parameters in the reference's ravel order: per block conv1.weight (C, Cin, 3, 3),
 * conv1.bias (C), conv2.weight (C, C, 3, 3), conv2.bias (C, absent in the last block);
 * Cin = 1 in block 0. Supported: L x L periodic lattices with L*L <= 256, C in {4,8,12,16}.
 * The complex_out argument of every ResConv entry point holds flags: QGX_RESCONV_COMPLEX,
 * complex output (pair_cpl: the first C/2 channels are the real part), and QGX_RESCONV_SINHP1,
 * the final activation sinhp1_by_scale, psi = mean (sinh z + 1), instead of exp_by_scale,
 * psi = mean exp z (nn/activation.py:7-32). A real sinhp1 state can be negative: its log psi
 * carries the sign as the phase 0 or pi. */
#define QGX_RESCONV_COMPLEX 1
#define QGX_RESCONV_SINHP1 2
int64_t qgx_resconv_nparams(int32_t nblocks, int32_t channels);
int64_t qgx_resconv_table_floats(int32_t nblocks, int32_t channels);
/* Convolution arithmetic of the forward pass (log_psi, sweep, eloc). FP32: CUDA-core FMA
 * in FP32. TF32 / BF16: the 3x3 convolutions of blocks run as tcgen05 MMAs with TF32 or
 * BF16 operands and FP32 accumulation (residual stream, GELU, biases and the log-sum-exp
 * stay FP32; the first, one-channel convolution stays on the CUDA cores). The tensor-core
 * forms take C <= 16 (run padded to 16 channels) and L <= 16. */
#define QGX_CONV_FP32 0
#define QGX_CONV_TF32 1
#define QGX_CONV_BF16 2
/* OR'd into QGX_CONV_BF16: run the warp-specialised tensor-core kernel (one CTA per SM with
 * three sample groups, one MMA warp serving them as their inputs become ready, all layers'
 * weights resident) instead of the default per-layer-synchronous one (three CTAs per SM, each
 * issuing a layer's MMAs and then running its epilogue). Both give bit-identical results; on
 * GB300 the grouped kernel is slower (1.13 against 0.82 ms for 16384 forwards at L = 10,
 * 8 blocks, 16 channels): one issuing thread takes about 115 clocks per N = 16 MMA, three
 * CTAs issuing side by side about 47. */
#define QGX_CONV_GROUPED 0x100
/* Reorder the parameters into the kernels' table (FP32 layers, then the BF16 and TF32
 * weight images of the tensor-core forward); re-run after every parameter update. */
int qgx_resconv_prepare(const float* params, int32_t nblocks, int32_t channels, float* table,
                        qgx_stream_t stream);
/* log psi(s) as (re, im) float pairs (2*ns floats); im = 0 for real output
 * (Variational.__call__, quantax/state/variational.py:325-347). */
int qgx_resconv_log_psi(const float* table, int32_t L, int32_t nblocks, int32_t channels,
                        int32_t complex_out, int32_t conv_precision, const uint32_t* spins, int64_t ns, float* log_psi,
                        qgx_stream_t stream);
int64_t qgx_resconv_sweep_workspace_bytes(int32_t L, int64_t ns);
/* nsteps SpinExchange proposals per chain (common_samplers.py:58-162, metropolis.py:246-322):
 * each step proposes for every chain, evaluates the proposals with one batched forward and
 * accepts in log space on the shared Philox stream. log_psi: (re, im) pairs, in/out
 * (recomputed at the start). */
int qgx_resconv_sweep(const float* table, int32_t L, int32_t nblocks, int32_t channels,
                      int32_t complex_out, int32_t conv_precision, uint32_t* spins, float* log_psi, int32_t* accepts,
                      int64_t ns, int32_t nsteps, uint64_t seed, uint64_t step0, float reweight,
                      const int32_t* nbr, int32_t z, int32_t hop, void* workspace,
                      int64_t workspace_bytes, qgx_stream_t stream);
/* max_conn = n_f1 + n_f2 of the operator. */
int64_t qgx_resconv_eloc_workspace_bytes(int32_t L, int64_t ns, int32_t max_conn);
/* Complex local energies over the compacted connected configurations (Operator.Oloc,
 * quantax/operator/operator.py:510-562, with the nonzero compaction of :144-165);
 * eloc_im may be NULL for real output. */
int qgx_resconv_eloc(const float* table, int32_t L, int32_t nblocks, int32_t channels,
                     int32_t complex_out, int32_t conv_precision, const qgx_operator_t* op, const uint32_t* spins, int64_t ns,
                     double* eloc_re, double* eloc_im, void* workspace, int64_t workspace_bytes,
                     qgx_stream_t stream);

/* Workspace bytes of qgx_resconv_jacobian (per-CTA activation scratch). */
int64_t qgx_resconv_jacobian_workspace_bytes(int32_t L, int32_t nblocks, int32_t channels);
/* Per-sample log-derivatives by a hand-written backward pass: O_re = d Re log psi / d params,
 * O_im = d Im log psi / d params (complex output; may be NULL for real output), row stride
 * ldo floats, parameter order as qgx_resconv_prepare (Variational.jacobian,
 * quantax/state/variational.py:424-511, VS_TYPE real_to_complex :40-94). Passing
 * O_im = O_re + ns * ldo writes the stacked [Re; Im] matrix of QNGD.solve (sr.py:99-105). */
int qgx_resconv_jacobian(const float* table, int32_t L, int32_t nblocks, int32_t channels,
                         int32_t complex_out, const uint32_t* spins, int64_t ns, float* O_re,
                         float* O_im, int64_t ldo, void* workspace, int64_t workspace_bytes,
                         qgx_stream_t stream);

/* ---- symmetry projection (Variational(symm=...), quantax/state/variational.py:261-266,
 * quantax/symmetry/symmetry.py:325-392) --------------------------------------------------
 * psi_symm(s) = sum_g w_g psi(T_g s) with w_g = chi_0 chi_g / |G|. T_g s for g < nperm puts
 * s[perm[g * N + i]] at site i (Symmetry.get_symm_spins); with z2 != 0 the elements
 * nperm .. 2 nperm - 1 are the same permutations of -s, weighted by z2 chi (Z2 inversion).
 * weight: (re, im) of w_g for g < nsymm = nperm (z2 ? 2 : 1), device doubles.
 * The forward evaluates every T_g s with the same kernels as the unsymmetrised entry points
 * and combines the |G| values per configuration in log space; a configuration whose sum
 * vanishes gets log |psi| = -inf. */
typedef struct {
  const int16_t* perm;   /* device, nperm x N */
  const double* weight;  /* device, 2 * nsymm */
  int32_t nperm;
  int32_t z2;            /* 0, 1 or -1 (only its being non-zero is read here) */
} qgx_symm_t;

int64_t qgx_resconv_log_psi_symm_workspace_bytes(int32_t L, int64_t ns, int32_t nsymm);
int qgx_resconv_log_psi_symm(const float* table, int32_t L, int32_t nblocks, int32_t channels,
                             int32_t complex_out, int32_t conv_precision, const qgx_symm_t* symm,
                             const uint32_t* spins, int64_t ns, float* log_psi, void* workspace,
                             int64_t workspace_bytes, qgx_stream_t stream);
int64_t qgx_resconv_sweep_symm_workspace_bytes(int32_t L, int64_t ns, int32_t nsymm);
/* qgx_resconv_sweep for the symmetrised state: log_psi holds log psi_symm. */
int qgx_resconv_sweep_symm(const float* table, int32_t L, int32_t nblocks, int32_t channels,
                           int32_t complex_out, int32_t conv_precision, const qgx_symm_t* symm,
                           uint32_t* spins, float* log_psi, int32_t* accepts, int64_t ns, int32_t nsteps,
                           uint64_t seed, uint64_t step0, float reweight, const int32_t* nbr, int32_t z,
                           int32_t hop, void* workspace, int64_t workspace_bytes, qgx_stream_t stream);
int64_t qgx_resconv_eloc_symm_workspace_bytes(int32_t L, int64_t ns, int32_t max_conn, int32_t nsymm);
int qgx_resconv_eloc_symm(const float* table, int32_t L, int32_t nblocks, int32_t channels,
                          int32_t complex_out, int32_t conv_precision, const qgx_symm_t* symm,
                          const qgx_operator_t* op, const uint32_t* spins, int64_t ns, double* eloc_re,
                          double* eloc_im, void* workspace, int64_t workspace_bytes, qgx_stream_t stream);
int64_t qgx_resconv_jacobian_symm_workspace_bytes(int32_t L, int32_t nblocks, int32_t channels, int64_t ns,
                                                  int32_t nsymm);
/* d log psi_symm / d params = sum_g v_g d log psi(T_g s) / d params with v_g = w_g psi(T_g s) /
 * psi_symm(s) (the cotangents of variational.py:441-477): one backward per group element,
 * seeded with v_g, accumulated into the sample's row. v_g comes from an FP32 forward. */
int qgx_resconv_jacobian_symm(const float* table, int32_t L, int32_t nblocks, int32_t channels,
                              int32_t complex_out, const qgx_symm_t* symm, const uint32_t* spins, int64_t ns,
                              float* O_re, float* O_im, int64_t ldo, void* workspace,
                              int64_t workspace_bytes, qgx_stream_t stream);

/* The projected RBM_Dense (Variational(RBM_Dense, symm=...): the reference projects any model,
 * quantax/state/variational.py:261-266). The table is qgx_rbm_prepare's; n <= 256 sites,
 * m <= 2048 hidden units. Every T_g s runs through the RBM's own forward and closed-form
 * log-derivatives; the projection itself is the ResConv entry points' pipeline. log_psi holds
 * (re, im) pairs: psi_symm is complex for complex characters and signed for real ones. */
int64_t qgx_rbm_log_psi_symm_workspace_bytes(int32_t n, int64_t ns, int32_t nsymm);
int qgx_rbm_log_psi_symm(const float* table, int32_t n, int32_t m, const qgx_symm_t* symm,
                         const uint32_t* spins, int64_t ns, float* log_psi, void* workspace,
                         int64_t workspace_bytes, qgx_stream_t stream);
int64_t qgx_rbm_sweep_symm_workspace_bytes(int32_t n, int64_t ns, int32_t nsymm);
/* Metropolis sweep of the projected RBM (metropolis.py:246-322): per step every chain
 * proposes (LocalFlip: one uniform site, Philox word 0; SpinExchange as qgx_rbm_sweep, nbr may
 * be NULL for LocalFlip), the changed proposals are evaluated as one projected batch and
 * accepted in log space on the shared Philox stream. log_psi: (re, im) pairs, out. */
int qgx_rbm_sweep_symm(const float* table, int32_t n, int32_t m, const qgx_symm_t* symm, uint32_t* spins,
                       float* log_psi, int32_t* accepts, int64_t ns, int32_t nsteps, uint64_t seed,
                       uint64_t step0, float reweight, int32_t proposal, const int32_t* nbr, int32_t z,
                       int32_t hop, void* workspace, int64_t workspace_bytes, qgx_stream_t stream);
int64_t qgx_rbm_eloc_symm_workspace_bytes(int32_t n, int64_t ns, int32_t max_conn, int32_t nsymm);
/* E_loc of the projected RBM (operator.py:510-562): eloc_im may be NULL for real characters. */
int qgx_rbm_eloc_symm(const float* table, int32_t n, int32_t m, const qgx_symm_t* symm,
                      const qgx_operator_t* op, const uint32_t* spins, int64_t ns, double* eloc_re,
                      double* eloc_im, void* workspace, int64_t workspace_bytes, qgx_stream_t stream);
int64_t qgx_rbm_jacobian_symm_workspace_bytes(int32_t n, int32_t m, int32_t has_vbias, int64_t ns,
                                              int32_t nsymm);
/* d log psi_symm / d params = sum_g v_g O(T_g s), v_g = w_g psi(T_g s) / psi_symm(s): the images'
 * closed-form O rows (qgx_rbm_jacobian's) combined per sample in FP32, Re to O_re, Im to O_im
 * (may be NULL), parameter order as qgx_rbm_jacobian. */
int qgx_rbm_jacobian_symm(const float* table, int32_t n, int32_t m, int32_t has_vbias, const qgx_symm_t* symm,
                          const uint32_t* spins, int64_t ns, float* O_re, float* O_im, int64_t ldo,
                          void* workspace, int64_t workspace_bytes, qgx_stream_t stream);

/* ---- statistics and centring (quantax/optimizer/sr.py:76-88, 180-195) ----------------- */
/* energy = Re mean(E r), VarE = mean(|E - energy|^2 r) with compensated FP64 sums;
 * ebar = (E - mean E) sqrt(r / ns). E_im / ebar_im may be NULL for real E.
 * stats[0..2] = {Re energy, Im energy, VarE}. */
int qgx_energy_stats(const double* E_re, const double* E_im, const double* r, int64_t ns,
                     double* stats, double* ebar_re, double* ebar_im, qgx_stream_t stream);
/* Consistency of log|psi| carried through local updates with a direct forward
 * (Metropolis.sweep, quantax/sampler/metropolis.py:201-213): *count (device int) = number of
 * samples for which neither |psi_l - psi_d| < 1e-8 nor |psi_l / psi_d - 1| < 1e-3 holds;
 * out (may be NULL or equal local) receives the direct values, which replace the local ones
 * as in the reference. */
int qgx_log_psi_mismatch(const float* local, const float* direct, int64_t ns, int32_t* count,
                         float* out, qgx_stream_t stream);
/* Reweight factors r_s = |psi_s|^(2-n) / mean (Sampler._get_reweight_factor,
 * quantax/sampler/sampler.py:66-69), from log|psi|. */
int qgx_reweight_factor(const float* log_psi, int64_t ns, float reweight, double* r,
                        qgx_stream_t stream);
/* Workspace bytes of qgx_center_columns. */
int64_t qgx_center_columns_workspace_bytes(int64_t ns, int64_t np);
/* In-place O -> (O - mean_s O) * sqrt(r_s / ns) for a dense (ns x np) matrix, and
 * omean = mean_s(O r). Generic form of the centring used by non-RBM models. */
int qgx_center_columns(float* O, int64_t ns, int64_t np, int64_t ldo, const double* r,
                       double* omean, void* workspace, int64_t workspace_bytes,
                       qgx_stream_t stream);

/* ---- momentum variants of SR (SPRING, MARCH, AdamSR: quantax/optimizer/sr.py:198-429) --- */
/* y = A x for the FP32 Obar A (rows x cols, row stride lda floats), FP64 x and y. */
int qgx_obar_matvec(const float* A, int64_t rows, int64_t cols, int64_t lda, const double* x,
                    double* y, qgx_stream_t stream);
/* A[:, j] *= s[j] in place (FP64 scale factors). */
int qgx_scale_columns(float* A, int64_t rows, int64_t cols, int64_t lda, const double* s,
                      qgx_stream_t stream);

/* ---- exact sampling (ExactSampler, quantax/sampler/sampler.py:72-119) ------------------ */
/* idx[i] (i < ns) = the first j with cdf[j] > u_i cdf[dim - 1], cdf the inclusive prefix sums
 * of the probabilities of a basis (dim doubles, cdf[dim - 1] > 0), u_i in [0, 1) the 53-bit
 * uniform of Philox draw (seed, counter (i, step, tag 4)). Replaces jr.choice(..., p=prob) of
 * ExactSampler.sweep (sampler.py:108-110). */
int qgx_exact_draw(const double* cdf, int64_t dim, int64_t ns, uint64_t seed, uint64_t step,
                   int64_t* idx, qgx_stream_t stream);

/* ---- exact reconfiguration (ER, quantax/optimizer/sr.py:432-513) over a whole basis ---- */
/* y = H x for a CSR matrix (nrows x nrows; rowptr nrows + 1 int64, col int32, val FP64):
 * nvec = 1 for real x, y (nrows doubles), 2 for complex ones as (re, im) pairs. Replaces the
 * QuSpin product `hamiltonian @ DenseState` of ER.get_Ebar (sr.py:488-495). */
int qgx_csr_matvec(const int64_t* rowptr, const int32_t* col, const double* val, int64_t nrows,
                   const double* x, int nvec, double* y, qgx_stream_t stream);
/* Omat = psi_s O_s in place, a NaN product set to 0 (ER.get_Obar, sr.py:497-505). cplx = 0:
 * O (ns x cols, row stride ldo floats), psi ns doubles; cplx = 1: O holds [Re O; Im O]
 * (2 ns rows), psi ns (re, im) pairs. */
int qgx_er_weight_rows(float* O, int64_t ns, int64_t cols, int64_t ldo, const double* psi, int cplx,
                       qgx_stream_t stream);
/* Obar = Omat - psi Omean^T in place, Omean = psi^H Omat (cols doubles, or cols real parts then
 * cols imaginary parts when cplx = 1). */
int qgx_er_center(float* O, int64_t ns, int64_t cols, int64_t ldo, const double* psi, int cplx,
                  const double* omean, qgx_stream_t stream);

/* ---- Gram matrices (quantax/optimizer/solver.py:139, 157) ---------------------------- */
/* T = A A^T for A (rows x k, row stride lda floats), written as FP64 rows x rows
 * (full symmetric matrix, row stride ldt). mode = QGX_GRAM_*. */
int qgx_gram(const float* A, int64_t rows, int64_t k, int64_t lda, double* T, int64_t ldt,
             int32_t mode, qgx_stream_t stream);
/* T = A A^T on the tcgen05 tensor cores: A is FP32 read as TF32 (a_dtype 0), bf16
 * (a_dtype 1) or FP32 split in-kernel into TF32 hi + lo parts with T = hi hi^T + hi lo^T +
 * lo hi^T (a_dtype 2, FP32-class accuracy); FP32 accumulation in TMEM, T written as FP64
 * (full symmetric matrix).
 * Needs k > 0, a 16-byte aligned A and lda * element size a multiple of 16 bytes (else
 * QGX_ERR_UNSUPPORTED). status (device int, may be NULL) is set to QGX_ERR_TIMEOUT if a
 * bounded pipeline wait expired, else 0. */
int qgx_gram_tc(const void* A, int32_t a_dtype, int64_t rows, int64_t k, int64_t lda, double* T,
                int64_t ldt, int32_t* status, qgx_stream_t stream);
/* bf16 copy of an FP32 matrix (round to nearest even), the operand of the bf16 Gram. */
int qgx_f32_to_bf16(const float* in, int64_t rows, int64_t k, int64_t ldi, uint16_t* out,
                    int64_t ldo, qgx_stream_t stream);
/* out = A^T (cols x rows, row stride ldo elements) of an FP32 matrix (rows x cols, ldi);
 * out_dtype 0: FP32, 1: BF16 (round to nearest even). With it the tensor-core Gram computes
 * the SR branch's S = A^T A as the Gram of A^T (rows <= 2097120). */
int qgx_transpose(const float* in, int64_t rows, int64_t cols, int64_t ldi, void* out, int64_t ldo,
                  int32_t out_dtype, qgx_stream_t stream);
/* S = A^T A (k x k) for the SR branch (Ns >= Np), FP32 on the CUDA cores. */
int qgx_gram_t(const float* A, int64_t rows, int64_t k, int64_t lda, double* S, int64_t lds,
               qgx_stream_t stream);

/* ---- FP64 solve (quantax/optimizer/solver.py:50-201) -------------------------------- */
/* Workspace bytes of qgx_minsr_solve (Gram n x n, A n x np) or qgx_sr_solve (Gram
 * np x np, pass n = np of the Gram and np = the number of samples). */
int qgx_solve_workspace_bytes(int64_t n, int64_t np, int32_t method, int64_t* bytes);
/* MinSR branch: given T = A A^T (n x n FP64, overwritten), b (n), A (n x np FP32):
 *   SHIFT: (T + (rshift tr T + ashift) I) y = b by Cholesky, x = A^T y
 *   PINV:  T = U diag(l) U^T, x = A^T U diag(l+) rho, rho = sum_without_noise(U^T o b)
 *   SHIFT_MIXED: as SHIFT; FP64 conjugate gradients preconditioned by the FP32 Cholesky factor
 *                (see QGX_SOLVE_SHIFT_MIXED); synchronises the stream with the host
 * x (np doubles). info (device int, may be NULL) receives the cuSOLVER info: > 0 the
 * shifted matrix is not positive definite at that leading minor (x is then NaN, like the
 * reference's Cholesky solve); -1 the mixed-precision refinement did not converge (x holds
 * the last iterate; factor the shifted T, still in place, with SHIFT and zero shifts). */
int qgx_minsr_solve(double* T, int64_t n, const float* A, int64_t np, int64_t lda,
                    const double* b, int32_t method, double rshift, double ashift,
                    double rtol, double atol, double tol_snr, double* x, int32_t* info,
                    void* workspace, int64_t workspace_bytes, qgx_stream_t stream);
/* Number of qgx kernels the last qgx_minsr_solve / qgx_sr_solve call of this host thread
 * launched (library kernels such as cuSOLVER's not counted; SHIFT_MIXED varies with its
 * iteration count). */
int64_t qgx_last_solve_kernels(void);
/* SR branch: given S = A^T A (np x np FP64, overwritten): x = S^-1 A^T b with the same
 * two regularisations (lstsq_shift_eig / lstsq_pinv_eig). PINV with tol_snr > 1e-6 applies
 * lstsq_pinv_eig's noise truncation (solver.py:152-164 with _sum_without_noise, :114-125):
 * rho_k = sum_s t_sk / (1 + (tol_snr / snr_k)^6) over the per-sample terms
 * t_sk = b_s (A V)_sk, snr_k = |mean_s t_sk| / sqrt(var_s t_sk / n). */
int qgx_sr_solve(double* S, int64_t np, const float* A, int64_t n, int64_t lda,
                 const double* b, int32_t method, double rshift, double ashift,
                 double rtol, double atol, double tol_snr, double* x, int32_t* info,
                 void* workspace, int64_t workspace_bytes, qgx_stream_t stream);

/* FP64 Cholesky factorisation A = L L^T of a symmetric positive definite n x n matrix
 * (row-major, leading dimension lda; the factor step of minnorm_shift_eig / lstsq_shift_eig,
 * quantax/optimizer/solver.py:50-91, jax.scipy.linalg.solve(assume_a="pos")). L overwrites the
 * lower triangle (L[i][j] at A[i lda + j], i >= j); the strict upper triangle keeps the input.
 * Read as column-major, the result is the upper factor U = L^T (A = U^T U) that cuSOLVER's
 * potrs takes with CUBLAS_FILL_MODE_UPPER. 64 x 64 diagonal blocks and their triangular solves
 * run in FP64; every update C -= P P^T (P a 64- or 256-column panel) runs on the tensor cores
 * as an exact product of 8 BF16 digit slices per element (row-scaled 57-bit fixed point,
 * integer accumulation exact in FP32), folded in int64 and applied in FP64.
 * info (device int): 0, or the order of the first leading minor that is not positive
 * definite. status (device int, may be NULL): QGX_ERR_TIMEOUT if a tensor-core wait ran out
 * (the factor is then invalid). Workspace: qgx_cholesky_workspace_bytes(n), 256-byte
 * aligned; no counterpart in the reference beyond the factorisation it calls. */
int64_t qgx_cholesky_workspace_bytes(int64_t n);
int qgx_cholesky(double* A, int64_t n, int64_t lda, int32_t* info, int32_t* status,
                 void* workspace, int64_t workspace_bytes, qgx_stream_t stream);

/* Real-time evolution's S-path (quantax/optimizer/time_evol.py:55-134):
 * y = A^T b (cols doubles), FP64 accumulation in a fixed order; workspace from
 * qgx_obar_rmatvec_workspace_bytes. */
int qgx_obar_rmatvec_workspace_bytes(int64_t rows, int64_t cols, int64_t* bytes);
int qgx_obar_rmatvec(const float* A, int64_t rows, int64_t cols, int64_t lda, const double* b,
                     double* y, void* workspace, int64_t workspace_bytes, qgx_stream_t stream);
/* out[col] = sum over rows of A[row][col]^2 (diag(A^T A)), about 48-bit sums; workspace from
 * qgx_column_sumsq_workspace_bytes (lstsq_shift_cg's relative shift, solver.py:24-47). */
int64_t qgx_column_sumsq_workspace_bytes(int64_t rows, int64_t cols);
int qgx_column_sumsq(const float* A, int64_t rows, int64_t cols, int64_t lda, double* out,
                     void* workspace, int64_t workspace_bytes, qgx_stream_t stream);
/* x = S^-1 f for a symmetric S (n x n FP64, overwritten): PINV is pinvh_solve
 * (solver.py:104-111, eigh with the soft inverse), SHIFT the shifted Cholesky solve.
 * Workspace: qgx_solve_workspace_bytes(n, 1, method). */
int qgx_sym_solve(double* S, int64_t n, const double* f, int32_t method, double rshift,
                  double ashift, double rtol, double atol, double* x, int32_t* info,
                  void* workspace, int64_t workspace_bytes, qgx_stream_t stream);

/* ---- parameter update (quantax/state/variational.py:558-579) ------------------------- */
/* params <- params - step when every step entry is finite; otherwise params are left
 * unchanged and *flag (device int) is set to 1 (else 0). */
int qgx_apply_update(float* params, const double* step, int64_t np, int32_t* flag,
                     qgx_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* QGX_H_ */
