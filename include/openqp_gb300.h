/*
 * openqp_gb300 -- GB300-native direct two-electron Fock (J/K) build for OpenQP.
 *
 * C ABI of libopenqp_gb300.so.  Plain pointers and sizes only; every pointer
 * is host memory unless the name says _device.  All entry points return (or
 * store in *info) an OpenQP route-C status code:
 *   0 success, 1 not initialised, 2 out of memory, 3 unsupported input
 *   (angular momentum above f, mixed Cartesian/pure d and f shells), 4 device
 *   error.  A non-zero status means the caller's native path must run, which
 *   is exactly the contract of OpenQP's seam (source/modules/routec_bridge.F90:20-22).
 *
 * Two layers:
 *   - routec_*: the reference-facing seam.  routec_fock_jk has the signature
 *     OpenQP binds by dlopen/dlsym or at link time
 *     (source/modules/routec_bridge.F90:33-40, 81-89, 204-216); it works on a
 *     process-global context registered once by routec_fock_init.
 *   - oqpg_*: an explicit-context API (several molecules at once, device
 *     pointers, CUDA streams) used by the Python/torch front end and the
 *     batched builds.
 *
 * Matrices are OpenQP's packed lower triangles, row-major with
 * ij = i(i+1)/2 + j (0-based, i >= j), stacked per density:
 *   d[nfocks][nbf(nbf+1)/2], f[nfocks][nbf(nbf+1)/2].
 * nfocks = 1: RHF, F = sc J[D] - se/2 K[D];
 * nfocks = 2: UHF/ROHF, F_s = sc J[Da + Db] - se K[D_s]
 * (source/integrals/int2.F90:1414-1578 with the scaling of
 *  source/scf_addons.F90:1177-1185 folded in: f comes back ready to use).
 */
#ifndef OPENQP_GB300_H
#define OPENQP_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- reference-facing seam ------------------------------------------- */

/* Register the basis and geometry used by the following routec_fock_jk
 * calls, in the layout of OpenQP's basis_set (source/basis_tools.F90:32-84):
 *   am[nshell], ncontr[nshell], origin[nshell] (1-based atom), harmonic[nshell]
 *   (1 = pure spherical shell), ex/cc[sum ncontr] (cc primitive-normalised,
 *   as after basis%normalize_primitives, source/basis_tools.F90:277-303),
 *   xyz[3*natom] in Bohr, cutoff = OpenQP's int2e_cutoff (source/types.F90:121).
 * Computes the Schwarz bounds on the device (ints_exchange,
 * source/integrals/int2.F90:1582-1737).  There is no counterpart in the
 * reference seam, which carries no basis (routec_bridge.F90:33-40); OpenQP
 * would call this next to scf_addons.F90:1141.  Returns a status code. */
int routec_fock_init(int nshell, const int* am, const int* ncontr, const int* origin, const double* ex,
                     const double* cc, const int* harmonic, int natom, const double* xyz, double cutoff);

/* The seam itself: replaces fock_jk's native int2 path
 * (source/scf_addons.F90:1138-1146, routec_bridge.F90:33-40).  All arguments
 * by reference, Fortran style.  f is overwritten. */
void routec_fock_jk(const double* d, double* f, const int* nbf, const int* nfocks, const double* se,
                    const double* sc, int* info);

/* Incremental build F = F_old + G(D - D_old), F_old <- F: the branch of fock_jk
 * taken when f_old is present (source/scf_addons.F90:1207-1210, 2036-2043),
 * which the reference seam declines (scf_addons.F90:1141).  dd = D - D_old. */
void routec_fock_jk_inc(const double* dd, double* f, double* f_old, const int* nbf, const int* nfocks,
                        const double* se, const double* sc, int* info);

/* Batched builds (many molecules in one build, one captured CUDA graph):
 * register nmol molecules on the process-global context, then build all their
 * Fock matrices in one call.  Arguments as oqpg_create_batch; d and f are the
 * molecules' packed matrices one after the other (layout of oqpg_fock_jk on a
 * batch context).  routec_fock_jk_batch checks *nmol against the registered
 * batch.  No counterpart in the reference, which builds one molecule per
 * fock_jk call. */
int routec_fock_init_batch(int nmol, const int* nshell, const int* natom, const int* am, const int* ncontr,
                           const int* origin, const double* ex, const double* cc, const int* harmonic,
                           const double* xyz, double cutoff);
void routec_fock_jk_batch(const double* d, double* f, const int* nmol, const int* nfocks, const double* se,
                          const double* sc, int* info);

/* Precision split of the following builds on the process-global context
 * (see oqpg_set_precision).  No counterpart in the reference seam. */
int routec_fock_set_precision(int mode, double threshold);

/* Run-time two-electron cutoff of the following builds on the process-global
 * context (oqpg_set_cutoff).  Replaces int2_compute_t_set_cutoff
 * (source/integrals/int2.F90:480-496): the progressive-screening SCF changes
 * infos%control%int2e_cutoff before every build (source/scf.F90:721-734) and
 * fock_jk re-reads it (int2.F90:271).  *cutoff > 0; *info = 0, 1 (not
 * initialised) or 3 (not a positive finite cutoff).  By reference, Fortran
 * style. */
void routec_fock_set_cutoff(const double* cutoff, int* info);

/* Petite list of the process-global context (oqpg_set_symmetry) from
 * OpenQP's own symmetry arrays, as pyoqp stages them for
 * int2_compute_t_enable_petite and symmetrize_skeleton_signed
 * (source/integrals/int2.F90:312-365, source/scf_addons.F90:1563-1615):
 * shell_map[(op-1)*nshell + s] and ao_target[(op-1)*nbf + mu] the 1-based
 * images of shell s and AO mu under operation op (integer(8), tagarrays
 * OQP_sym_shell_map, OQP_sym_ao_target), ao_sign[(op-1)*nbf + mu] = +-1
 * (OQP_sym_ao_sign).  *nops <= 1 switches the reduction off.  The seam still
 * returns the complete Fock matrix.  *info = 0, 1 (not initialised) or 3
 * (not an abelian group of signed AO permutations of this basis).  All
 * arguments by reference, Fortran style. */
void routec_fock_set_symmetry(const int* nops, const long long* shell_map, const long long* ao_target,
                              const double* ao_sign, int* info);

/* The reference's 2e-gradient seam (source/modules/routec_bridge.F90:51-61,
 * 241, 292-310; caller source/modules/hf_gradient.F90:270-289): d is the
 * packed total RHF density, xyz(3, natm) in Bohr must be the geometry
 * registered by routec_fock_init, de(3, natm) is ACCUMULATED with dE2e/dR
 * (Coulomb scaled by coulscale, exchange by hfscale).  All arguments by
 * reference.  Declines (info = 1) for another basis or geometry. */
void routec_grad2(const double* d, const double* xyz, double* de, const int* nbf, const int* natm,
                  const double* hfscale, const double* coulscale, int* info);

/* routec_grad2_mrsf: the reference's MRSF gradient seam
 * (source/modules/routec_bridge.F90:65-76, called from
 * modules/tdhf_mrsf_gradient.F90:274-297 for non-CAM runs): oqpg_grad2_mrsf
 * on the routec_fock_init context, de(3, natm) accumulated; declines
 * (info = 1) for another basis or geometry. */
void routec_grad2_mrsf(const double* d, const double* p, const double* spc, const double* xyz, double* de,
                       const int* nbf, const int* natm, const double* hfscale, const double* hfscale2,
                       const double* coulscale, const double* spcscale, const int* mrst, int* info);

/* Response-type builds on the process-global context (extensions: the
 * reference has no seam for these digestions; a maintainer binds them in
 * place of the int2_driver%run call of the consumer).
 *
 * routec_fock_td replaces int2_td_data_t (source/tdhf_lib.F90:140-224 and its
 * parallel_stop :89-111), used by modules/tdhf_energy.F90:221,
 * modules/cphf.F90:193 and modules/nmr_shielding.F90:454-487.
 * d2(nbf, nbf, nvec) general square densities, apb / amb (nbf, nbf, nvec)
 * OVERWRITTEN, all Fortran column-major; flags = OQPG_TD_* (the data type's
 * int_apb, int_amb, tamm_dancoff, tamm_dancoff_coulomb); se / sc the
 * scale_exchange / scale_coulomb of the data type.  Outputs that the flags
 * do not ask for come back zero, as the reference's zero-initialised arrays.
 *
 * routec_fock_mrsf replaces the first pass of int2_mrsf_data_t (nmat = 7,
 * source/tdhf_mrsf_lib.F90:218-333) or int2_umrsf_data_t (nmat = 11,
 * :337-426) with tamm_dancoff = .true.; d3 / f3 (nvec, nmat, nbf, nbf)
 * Fortran column-major, f3 OVERWRITTEN.  CAM builds: oqpg_fock_td_cam /
 * oqpg_fock_mrsf_cam. */
#define OQPG_TD_APB 1
#define OQPG_TD_AMB 2
#define OQPG_TD_TDA 4
#define OQPG_TD_TDA_COULOMB 8
void routec_fock_td(const double* d2, double* apb, double* amb, const int* nbf, const int* nvec, const int* flags,
                    const double* se, const double* sc, int* info);
void routec_fock_mrsf(const double* d3, double* f3, const int* nbf, const int* nvec, const int* nmat,
                      const double* se, const double* sc, int* info);

/* routec_fock_tdgrd replaces int2_tdgrd_data_t (source/tdhf_lib.F90:228-295,
 * the int2_td_data_t parallel_stop :89-111), used by the SF / MRSF Z-vector
 * solvers (modules/tdhf_sf_z_vector.F90:252,377,489,
 * modules/tdhf_mrsf_z_vector.F90:1009,1737).  d2(nbf, nbf, 2) the alpha /
 * beta densities, apb / amb (nbf, nbf, 2) OVERWRITTEN; flags OQPG_TD_APB /
 * OQPG_TD_AMB; amb(:,:,2) comes back zero as in the reference.  cam = NULL
 * for the plain build, else the five CAM values of routec_fock_jk_cam (the
 * int2_run_cam two-pass build the callers request for CAM functionals).
 *
 * routec_fock_rpagrd replaces int2_rpagrd_data_t (source/tdhf_lib.F90:
 * 1068-1322), used by the TDHF / TDDFT gradient
 * (modules/tdhf_z_vector.F90:341,484).  xpy(nbf, nbf, ldp, np),
 * xmy(nbf, nbf, ldm, nm), t(nbf, nbf, ldt, nt) (ld >= nspin; a count of 0
 * leaves the pointer unread), hpp(nbf, nbf, nspin, np) = H+[X+Y],
 * hpt(.., nt) = H+[T], hmm(.., nm) = H-[X-Y], OVERWRITTEN.  H+ is formed from
 * the symmetric part of its operand (every reference caller passes symmetric
 * matrices; for other operands the reference's own sum depends on its quartet
 * order); H- fills spin component 1 only.  The screening density covers
 * every ld component of xpy and xmy (both only when np > 0) and of t, as
 * the reference's init_screen does. */
void routec_fock_tdgrd(const double* d2, double* apb, double* amb, const int* nbf, const int* flags, const double* se,
                       const double* sc, const double* cam, int* info);
void routec_fock_rpagrd(const double* xpy, const int* ldp, const int* np, const double* xmy, const int* ldm,
                        const int* nm, const double* t, const int* ldt, const int* nt, const int* nspin, const int* nbf,
                        double* hpp, double* hpt, double* hmm, const double* se, const double* sc, const double* cam,
                        int* info);

/* MRSF Davidson sigma session: the reference's routec_sig seam
 * (source/modules/routec_sig.F90:1-140, driven by
 * modules/tdhf_mrsf_energy.F90:638-690), on the routec_fock_init context.
 *
 * routec_sig_init uploads the MO coefficients mo_a / mo_b and the MO Fock
 * matrices fmo_a / fmo_b (C^T F C, unpacked), all (nbf, nbf) Fortran
 * column-major, for nocca / noccb occupied alpha / beta orbitals (MRSF:
 * nocca = noccb + 2) and kind 1 (singlet) or 3 (triplet); returns 0 when the
 * session is ready (1: no context or another basis, 3: unsupported input).
 * routec_sig_set_scale sets the HF exchange scale (scale_exchange =
 * scale_coulomb of the int2_mrsf_data_t build; 1 by default).
 * routec_sig_iter maps bvec_mo(ntrial, nv_new) to sigma_mo(ntrial, nv_new) =
 * (A-B) X, ntrial = nocca (nbf - noccb), the native mrsfcbc -> int2 ->
 * mrsfmntoia + mrsfesum product (info 0 on success; any other value tells
 * the caller to fall back to its native path).  routec_sig_free ends the
 * session (routec_fock_init / routec_fock_finalize end it too).  The
 * integrals use the context's cutoff; the reference's native response
 * screens at max(SCF cutoff, 1e-8) (tdhf_mrsf_energy.F90:511-514). */
int routec_sig_init(const int* nbf, const double* mo_a, const double* mo_b, const double* fmo_a, const double* fmo_b,
                    const int* nocca, const int* noccb, const int* kind);
void routec_sig_set_scale(const double* s);
void routec_sig_iter(const double* bvec_mo, const int* nv_new, double* sigma_mo, int* info);
void routec_sig_free(void);
/* routec_sig_iter on device buffers (bvec(ntrial, nv), sigma(ntrial, nv)) and
 * the given stream (null: the context's); synchronises before it returns.
 * Returns the status routec_sig_iter puts in info. */
int oqpg_sig_iter_device(const double* bvec, int nv, double* sigma, void* stream);

/* CAM (range-separated) build of routec_fock_jk's packed densities, the
 * path the reference runs natively for CAM functionals
 * (source/scf_addons.F90:1136-1167 skips the seam for them): int2_run_cam
 * (source/integrals/int2.F90:538-584).  cam[5] = {alpha, beta, mu,
 * alpha_coulomb, beta_coulomb}: pass 1 over 1/r with scale_exchange = alpha,
 * scale_coulomb = alpha_coulomb (the reference's default 1); pass 2 over the
 * erf(mu r)/r operator with its own Schwarz bounds, scale_exchange = beta,
 * scale_coulomb = beta_coulomb (default 0); f = the sum, scaled as
 * routec_fock_jk's. */
void routec_fock_jk_cam(const double* d, double* f, const int* nbf, const int* nfocks, const double* cam,
                        int* info);

/* Release the process-global context (no counterpart in the reference, whose
 * int2 state lives in module variables for the life of the process). */
void routec_fock_finalize(void);

/* ---- explicit-context API -------------------------------------------- */
/* No counterpart in the reference: the oqpg_* entry points take an explicit
 * context instead of the routec_* seams' process-global one, and serve the
 * Python/torch front end (device buffers, caller streams), batches of
 * molecules, captured graphs, tuning and statistics. */

typedef struct oqpg_ctx oqpg_ctx;

/* Same arguments as routec_fock_init; *out receives a new context. */
int oqpg_create(oqpg_ctx** out, int nshell, const int* am, const int* ncontr, const int* origin,
                const double* ex, const double* cc, const int* harmonic, int natom, const double* xyz,
                double cutoff);
int oqpg_destroy(oqpg_ctx* ctx);

/* A context over a batch of nmol molecules built together: molecule m has
 * nshell[m] shells on natom[m] atoms; am/ncontr/origin/harmonic, ex/cc and xyz
 * are the molecules' arrays of routec_fock_init one after the other (origin
 * 1-based within its molecule).  Every build of the context builds all
 * molecules: its d and f hold, molecule after molecule, nfocks packed
 * triangles of that molecule's nbf.  Shell quartets never mix molecules; the
 * quartet lists of each class span the whole batch, so one class launch
 * serves all molecules.  All molecules must agree on Cartesian or pure d. */
int oqpg_create_batch(oqpg_ctx** out, int nmol, const int* nshell, const int* natom, const int* am,
                      const int* ncontr, const int* origin, const double* ex, const double* cc, const int* harmonic,
                      const double* xyz, double cutoff);

/* Per molecule: nbf[m] and tri0[m], the offset of its packed block in units of
 * nfocks triangle elements (its block starts at nfocks * tri0[m]).  Either
 * pointer may be null.  Returns the number of molecules. */
int oqpg_batch_info(const oqpg_ctx* ctx, int* nbf, long long* tri0);

/* Number of basis functions of a context (summed over a batch). */
int oqpg_nbf(const oqpg_ctx* ctx);

/* Fock build from host buffers (H2D and D2H copies included). */
int oqpg_fock_jk(oqpg_ctx* ctx, const double* d, double* f, int nfocks, double se, double sc);

/* Fock build on device buffers: d_device / f_device are packed matrices in
 * device memory, stream a cudaStream_t (0 = the context's own stream).
 * Nothing is copied to or from the host except the per-class quartet counts. */
int oqpg_fock_jk_device(oqpg_ctx* ctx, const double* d_device, double* f_device, int nfocks, double se,
                        double sc, void* stream);

/* A plain-FP64 build of the packed densities on device buffers (as
 * oqpg_fock_jk_device in precision mode 0, with fixed launch parameters: the
 * primitive-parallel head at 2^8 primitive quartets, no tuned grid caps)
 * for callers that cannot allocate device memory while they build Fock
 * matrices (a host whose own pool allocator owns all device memory, or a loop
 * that cannot take the device synchronisation of cudaMalloc/cudaFree).  It
 * calls no cudaMalloc, cudaFree or other allocating routine: every per-build
 * buffer lives in one static 24 MiB device array that each GPU loading the
 * library holds until exit.  It follows the context's cutoff
 * (oqpg_set_cutoff) but ignores its precision split and tuning
 * (oqpg_set_precision, oqpg_set_tuning): it always builds in FP64.
 * Limits: nbf <= 128 and nshell <= 128 (checked before any kernel runs), and
 * as many screened quartets as the rest of the array holds (two 8-byte
 * entries each, about 1.5 million at nbf = 128), which is known only after
 * the screening pass: those two limits return 5 with f_device untouched.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; under lazy module loading
 * (CUDA_MODULE_LOADING=LAZY, the default) that lookup may also load the
 * module and reserve the static array at that moment, so make the first call
 * before any stream capture and before a pool allocator claims the remaining
 * device memory.  All calls share the array and each clears what must start at
 * zero; calls that overlap on the GPU race on it.  A failing launch or copy
 * waits for the work already queued on the stream before it returns 4, so no
 * kernel of the failed call still uses the array.  The context itself
 * (read-only tables) comes from oqpg_create.  There is no counterpart of this
 * entry point in the reference. */
int oqpg_fock_jk_noalloc(oqpg_ctx* ctx, const double* d_device, double* f_device, int nfocks, double se,
                         double sc, void* stream);

/* The build of oqpg_fock_jk_device replayed from a CUDA graph.  The first
 * call (and any call after a change of nfocks, se, sc, precision split or
 * tuning) builds directly, then captures the whole device-driven build --
 * density screening, quartet lists, primitive-count sort, every class kernel,
 * finalize -- into one graph on the context's buffers, with list capacities
 * sized from that density plus headroom.  Later calls copy d_device into the
 * graph's input, replay it and copy its output to f_device, all on stream, then
 * wait for the stream: when the density screens in more quartets than a list
 * holds, the replay leaves its output alone, and the call builds directly and
 * recaptures.  No counterpart in the reference. */
int oqpg_fock_jk_graph(oqpg_ctx* ctx, const double* d_device, double* f_device, int nfocks, double se,
                       double sc, void* stream);

/* Graph captures and replays so far, and kernels in the captured graph. */
int oqpg_graph_info(const oqpg_ctx* ctx, int* captures, int* replays, int* kernels);

/* Per-class launch parameters, 55 entries each in the class order of
 * oqpg_class_l (null: leave unchanged): split_log2 -- quartets with
 * >= 2^split_log2 surviving primitive quartets run the primitive-parallel
 * kernel, one warp per quartet with the lanes on its primitives (64: never;
 * -1, the default: for thread-per-quartet lists of builds with at most 32
 * densities sized on the device from the list's own primitive-quartet
 * histogram, 6 to 8, lower for short lists whose heaviest quartets would
 * otherwise outlast the rest, 8 in builds with more densities; 4 for
 * warp-per-quartet ones); chunk -- quartets a warp takes per work grab in the thread-per-quartet
 * kernels (multiple of 32); ctas_per_sm -- grid cap per SM (0: as many as
 * fit).  The autotuner of the Python front end picks them.  No counterpart in
 * the reference. */
int oqpg_set_tuning(oqpg_ctx* ctx, const int* split_log2, const int* chunk, const int* ctas_per_sm);
int oqpg_get_tuning(const oqpg_ctx* ctx, int* split_log2, int* chunk, int* ctas_per_sm);

/* Kernel family per class (55 entries): the classes with 28..108 Cartesian
 * elements and no f shell have both a thread-per-quartet kernel (the block in
 * registers) and a warp-per-quartet one.  family[c] = 0 (default): thread
 * per quartet when the class's list holds at least 1024 quartets per SM
 * (enough to fill the GPU), else warp per quartet; 1: thread per quartet; 2:
 * warp per quartet.  Ignored for classes with one family.  available[c] (get)
 * = 1 thread per quartet, 2 warp per quartet, 3 both.  The autotuner searches
 * it.  No counterpart in the reference. */
int oqpg_set_kernel_family(oqpg_ctx* ctx, const int* family);
int oqpg_get_kernel_family(const oqpg_ctx* ctx, int* family, int* available);

/* Shell families (on by default): two s shells of one atom whose primitive
 * exponents are the same, or one's among the other's (the generally
 * contracted shells of cc-pVXZ sets, which OpenQP stores as separate
 * segmented shells) share their primitive integrals in the (ss|ss), (ss|sp),
 * (ss|sd), (ss|pp), (ss|pd), (sp|sp), (sp|sd) and (sp|pp) classes of SCF
 * builds in every precision mode (in the split a family quartet runs in
 * FP32 when every member quartet it lists is below the threshold, else in
 * FP64, or double-float in the df modes): one primitive
 * integral per family quartet, added to every member shell quartet with its
 * own contraction factors, primitive screens, quartet screen, element cutoff
 * and digestion, so the result is the reference's shell-by-shell sum.
 * on = 0 evaluates every shell quartet on its own.  info: on, and the family
 * pairs with more than one member shell pair (0: the basis has no shared
 * primitives).  No counterpart in the reference (int2.F90 loops over shell
 * quartets). */
int oqpg_set_shell_families(oqpg_ctx* ctx, int on);
int oqpg_shell_families_info(const oqpg_ctx* ctx, int* on, int* nshared);

/* Schwarz bounds sqrt(max |(ab|ab)|) per shell pair, nshell x nshell (host);
 * single-molecule contexts only. */
int oqpg_schwarz(const oqpg_ctx* ctx, double* q);

/* Precision split of the following builds.  mode 0: every quartet in FP64
 * (the plain path, default).  mode 1: quartets whose screening value (Schwarz
 * bound x shell density, as in OpenQP's quartet screen) is below threshold are
 * evaluated in FP32 -- Rys roots and weights still in FP64 -- and their FP32
 * partial J/K blocks are added into the FP64 accumulators.  mode 2: as mode 1
 * with the FP32 quartets' roots and weights in FP32 as well.  mode 3
 * ("df"): no split; every quartet is evaluated in double-float arithmetic
 * (pairs of FP32 numbers, ~44 significant bits, on the FP32 pipe): the
 * thread-per-quartet classes digest in FP64, the warp-per-quartet classes in
 * double-float; all blocks are added into the FP64 accumulators (threshold
 * ignored).  mode 4 ("mixed-df"): the split of mode 2 with the quartets above
 * the threshold in double-float instead of FP64.  The gradient follows modes
 * 1, 2 and 4 with FP32 below the threshold and FP64 above it.  No counterpart
 * in the reference. */
int oqpg_set_precision(oqpg_ctx* ctx, int mode, double threshold);

/* Cutoff tau of the following Fock-type builds: the quartet screen (tau), the
 * primitive-quartet screen (1e-4 tau squared against p + q), the primitive
 * pair screen (1e-4 tau) and the element cutoff (tau), as
 * int2_compute_t_set_cutoff (source/integrals/int2.F90:480-496) sets them; the
 * exponent cutoff (25 ln 10) and the Schwarz bounds do not change.  A cutoff
 * at or above the one the context was created with only shortens the
 * primitive-pair ranges; a tighter one rebuilds the pair tables.  Returns 0, 1
 * (null context) or 3 (not a positive finite cutoff).  oqpg_get_cutoff returns
 * the current cutoff (-1 for a null context). */
int oqpg_set_cutoff(oqpg_ctx* ctx, double cutoff);
double oqpg_get_cutoff(const oqpg_ctx* ctx);

/* Petite list (symmetry reduction) of the following SCF builds of a
 * single-molecule context: the petite-list path of OpenQP's int2_twoei
 * (source/integrals/int2.F90:411-469, 781-795) with the skeleton
 * symmetrisation of fock_jk (source/scf_addons.F90:1205, 1563-1615), abelian
 * groups.  nops (2, 4 or 8) operations, each a signed permutation of the AOs:
 * shell_map[op*nshell + s] = the shell that op maps shell s onto (same angular
 * momentum), ao_target[op*nbf + mu] = AO i of that shell for AO i of shell s,
 * ao_sign[op*nbf + mu] = +-1; 0-based.  The operations must form a group.  A
 * build computes one quartet per orbit, weighted by the orbit size, and
 * returns the projection of the skeleton matrix onto the totally symmetric
 * component: the complete Fock matrix.  Each build checks on the device that
 * its densities are invariant (max |P(D) - D| <= 1e-6 max |D|, as
 * petite_density_asymmetry, scf_addons.F90:1250-1274) and builds every
 * quartet otherwise.  Response, CAM, gradient and no-alloc builds ignore it.
 * nops <= 1 switches it off.  Returns 0, 1 (null context) or 3 (a batch
 * context, or maps that are not a group of signed AO permutations).
 * oqpg_symmetry_info: the group order (1 without) and whether the last direct
 * build used the reduction. */
int oqpg_set_symmetry(oqpg_ctx* ctx, int nops, const int* shell_map, const int* ao_target, const double* ao_sign);
int oqpg_symmetry_info(const oqpg_ctx* ctx, int* nops, int* reduced);

/* Statistics of the last build, up to n (<= 230) doubles:
 * [0] quartets computed, [1] primitive quartets, [2] list build ms,
 * [3] integral kernels ms, [4] total device ms, [5] nbf, [6] shell pairs,
 * [7 .. 62) quartets per class (la lb|lc ld) in the order of oqpg_class_l,
 * [62 .. 117) primitive quartets per class, [117 .. 172) kernel ms per class,
 * [172] kernels launched by the build, [173] FP32 quartets, [174] FP32
 * primitive quartets, [175 .. 230) the part of each class's kernel ms spent
 * in its FP32 launches (precision split). */
int oqpg_stats(const oqpg_ctx* ctx, double* out, int n);

/* One-electron integrals on the host for the SCF around the Fock build
 * (nbf x nbf, row-major, same AO order and normalisation as the Fock build):
 * which = 0 overlap S, 1 kinetic energy T, 2 nuclear attraction V of the
 * point charges charges[natom] at xyz.  Basis arguments as routec_fock_init.
 * Runs on host threads; needs no GPU.  OpenQP computes these in its own
 * one-electron module (omp_hst, source/integrals/int1.F90:147-268); this is no seam
 * replacement, only the set-up the SCF loop around the seam needs. */
int oqpg_one_electron(int nshell, const int* am, const int* ncontr, const int* origin, const double* ex,
                      const double* cc, const int* harmonic, int natom, const double* xyz, const double* charges,
                      int which, double* out);

/* Two-electron HF gradient of a single-molecule context, accumulated into
 * de[3*natom]: OpenQP's grd2 (source/integrals/grd2.F90:145-391) for the
 * packed densities d (nfocks = 1: total RHF density; nfocks = 2: alpha and
 * beta), two-particle density 4 coulscale D_ij D_kl - hfscale (D_ik D_jl +
 * D_il D_jk [+ spin-density terms]) (source/modules/hf_gradient.F90:427-575),
 * with its screens and cutoffs.  Derivative ERIs up to (fd|dd) on the GPU,
 * contracted on the fly, nothing stored. */
int oqpg_grad2(oqpg_ctx* ctx, const double* d, int nfocks, double hfscale, double coulscale, double* de);

/* The same contraction for a general symmetric bilinear two-particle density
 * of full nbf x nbf AO matrices (row-major):
 *   G = cj sym(X_ab Y_cd) - ckt sym(X_ac Y_bd + X_ad Y_bc) - cks (spin pair xs, ys),
 * sym = average over exchanging X and Y; xs/ys both null or both set.  With
 * X = Y = D it is the energy gradient; with X = the upstream matrix of a
 * Fock build and Y = D it is the geometry part of that build's adjoint.  No
 * counterpart in the reference. */
int oqpg_grad2_bilinear(oqpg_ctx* ctx, const double* x, const double* y, const double* xs, const double* ys,
                        double cj, double ckt, double cks, double* de);

/* Statistics of the last gradient: [0] quartets listed, [1] quartets
 * evaluated, [2] primitive quartets, [3] ms (lists + kernels), [4] quartets
 * listed for FP32 (precision split).  The gradient follows the context's
 * precision split (oqpg_set_precision): quartets whose Schwarz bound times the
 * bound of their two-particle density is below the threshold run in FP32 and
 * add into the FP64 gradient. */
int oqpg_grad_stats(const oqpg_ctx* ctx, double* out, int n);

/* Two-electron MRSF gradient, accumulated into de(3, natom): grd2 with the
 * two-particle density of grd2_mrsf_compute_data_t (source/modules/
 * tdhf_mrsf_gradient.F90:341-355, 404-601).  d, p (nbf, nbf, 2): the RAW alpha
 * / beta SCF and relaxed difference densities (the sum / difference of its
 * init is formed here); spc (7, nbf, nbf): the response densities bo2v,
 * bo1v, bco1, bco2, o21v, co12, ball (general, not symmetric), all Fortran
 * column-major; spcscale = {spc_coco, spc_ovov, spc_coov}; mrst 1 or 3.
 * FP64 whatever the precision mode. */
int oqpg_grad2_mrsf(oqpg_ctx* ctx, const double* d, const double* p, const double* spc, double hfscale,
                    double hfscale2, double coulscale, const double* spcscale, int mrst, double* de);

/* CAM two-electron gradients: grd2_driver's CAM branch
 * (source/integrals/grd2.F90:104-128).  Pass 1 uses the regular integrals
 * with coulscale 1 and the alpha exchange scales.  Pass 2 uses erf(mu r)/r
 * with coulscale 0, the beta scales, its own Schwarz bounds
 * (grd2.F90:247-248) and the attenuated primitive screens
 * (grd2_rys.F90:368-373).  de is accumulated.
 * oqpg_grad2_cam: packed SCF densities as in oqpg_grad2 (nfocks 1 or 2).
 * oqpg_grad2_mrsf_cam: the MRSF form with cam5 = {reference alpha,
 * reference beta, response alpha, response beta, mu}; the spin-pair terms
 * enter both passes, as in the reference. */
int oqpg_grad2_cam(oqpg_ctx* ctx, const double* d, int nfocks, double alpha, double beta, double mu, double* de);
int oqpg_grad2_mrsf_cam(oqpg_ctx* ctx, const double* d, const double* p, const double* spc, const double* cam5,
                        const double* spcscale, int mrst, double* de);

/* Two-electron SF-TDDFT gradient of grd2_sf_compute_data_t
 * (source/modules/tdhf_sf_gradient.F90:277-502; the reference has no seam
 * for it, a maintainer replaces the grd2_driver call of sf_2e_grad): d, p as
 * in oqpg_grad2_mrsf, v (nbf, nbf) the spin-flip transition density (Fortran
 * column-major, general); de(3, natom) accumulated.  The density is the MRSF
 * one with ball = v and the spin-pair coupling terms off. */
int oqpg_grad2_sf(oqpg_ctx* ctx, const double* d, const double* p, const double* v, double hfscale, double hfscale2,
                  double coulscale, double* de);

/* Response-type builds (single-molecule contexts; see routec_fock_td and
 * routec_fock_mrsf for the layouts and the reference routines).  Every
 * density is screened, evaluated and digested in one pass over the quartets:
 * the integrals are computed once for all nvec (x nmat) matrices.  The
 * _device forms take device pointers and run on the given stream (null: the
 * context's), synchronising before they return.  The context's precision
 * mode applies. */
int oqpg_fock_td(oqpg_ctx* ctx, const double* d2, double* apb, double* amb, int nvec, int flags, double se,
                 double sc);
int oqpg_fock_td_device(oqpg_ctx* ctx, const double* d2, double* apb, double* amb, int nvec, int flags, double se,
                        double sc, void* stream);
int oqpg_fock_mrsf(oqpg_ctx* ctx, const double* d3, double* f3, int nvec, int nmat, double se, double sc);
int oqpg_fock_mrsf_device(oqpg_ctx* ctx, const double* d3, double* f3, int nvec, int nmat, double se, double sc,
                          void* stream);

/* Gradient-side response builds (layouts in routec_fock_tdgrd /
 * routec_fock_rpagrd); cam = NULL or the five CAM values.  The _device forms
 * take device pointers and run on the given stream (null: the context's). */
int oqpg_fock_tdgrd(oqpg_ctx* ctx, const double* d2, double* apb, double* amb, int flags, double se, double sc,
                    const double* cam);
int oqpg_fock_tdgrd_device(oqpg_ctx* ctx, const double* d2, double* apb, double* amb, int flags, double se,
                           double sc, const double* cam, void* stream);
int oqpg_fock_rpagrd(oqpg_ctx* ctx, const double* xpy, int ldp, int np, const double* xmy, int ldm, int nm,
                     const double* t, int ldt, int nt, int nspin, double* hpp, double* hpt, double* hmm, double se,
                     double sc, const double* cam);
int oqpg_fock_rpagrd_device(oqpg_ctx* ctx, const double* xpy, int ldp, int np, const double* xmy, int ldm, int nm,
                            const double* t, int ldt, int nt, int nspin, double* hpp, double* hpt, double* hmm,
                            double se, double sc, const double* cam, void* stream);

/* CAM forms (see routec_fock_jk_cam for cam[5]).  The TD build's two passes
 * accumulate before the A+B symmetrisation, as the reference's
 * parallel_stop runs after the last pass; the MRSF pass 2 updates only the
 * last component (tdhf_mrsf_lib.F90:314-328, 409-420).  Incremental (f_old)
 * CAM builds are not offered. */
int oqpg_fock_jk_cam(oqpg_ctx* ctx, const double* d, double* f, int nfocks, const double* cam);
int oqpg_fock_jk_cam_device(oqpg_ctx* ctx, const double* d_device, double* f_device, int nfocks, const double* cam,
                            void* stream);
int oqpg_fock_td_cam(oqpg_ctx* ctx, const double* d2, double* apb, double* amb, int nvec, int flags,
                     const double* cam);
int oqpg_fock_mrsf_cam(oqpg_ctx* ctx, const double* d3, double* f3, int nvec, int nmat, const double* cam);

/* Angular momenta (la, lb, lc, ld) of class c (0 <= c < 55): classes 0-20 are
 * the s-d ones, 21-54 those with an f shell (FP64 kernels only; the precision
 * modes keep them in FP64). */
int oqpg_class_l(int c, int* l4);

/* FP64 FMA throughput of the current device (TFLOP/s, FMA = 2 flops) from an
 * FMA-chain probe kernel; the denominator of the kernels' FP64 roofline. */
int oqpg_measure_fp64_peak(int iters, double* tflops);

/* Accuracy check of the kernels' own arithmetic: for n FP64 arguments
 * x_device[i] (device memory; the kernels' range, positive normal numbers
 * with 2^-126 <= x < 2^128) writes out_device[6 i + 0 .. 5] = the library's
 * FP64 1/sqrt(x), CUDA's rsqrt(x), the library's FP64 1/x, IEEE 1.0 / x, and
 * the double-float 1/sqrt(x) and 1/x of the df precision mode (as FP64).
 * Synchronises the device.  No counterpart in the reference. */
int oqpg_math_check(const double* x_device, double* out_device, long long n);

#ifdef __cplusplus
}
#endif

#endif /* OPENQP_GB300_H */
