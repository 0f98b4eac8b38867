/* wfs_fno.h — C ABI of the Fourier-neural-operator surrogate kernels.
 *
 * The surrogate jumps K split steps at once: psi(t + K dt) ~ prior + FNO(psi(t), V),
 * where prior is a coarse split step of the same interval. The reference has no
 * learned propagator; these entry points serve the surrogate's training and
 * inference loop (wavefunctionsimpython_gb300/fno.py), which is the only caller.
 *
 * All pointers are device pointers; every call is asynchronous on `stream`
 * (a cudaStream_t, NULL = the legacy default stream) and returns WFS_OK or a
 * WFS_ERR_* code from wfs.h.
 *
 * Layout ("packed"): a field with C channels (C even) over B samples of an
 * N^3 grid is a complex64 array [B][C/2][N^3]; channel 2j is the real part and
 * channel 2j+1 the imaginary part of pair j. psi itself is a 2-channel packed
 * field. Pointwise weights are row-major [cout][cin] float32 with a float32
 * bias [cout].
 *
 * Spectral layer: S(h) = Re F^-1 [ R(k) . F(h)(k) on the kept modes, 0 elsewhere ]
 * with F the unitary 3D DFT (applied to each channel) and the kept modes
 * kx, ky in [0, m) u [N-m, N), kz in [0, m): nmodes = 4 m^3, ordered
 * mode = (ix * 2m + iy) * m + iz. Mode-major activations are complex64
 * [nmodes][B][C]; weights are complex float32 R[nmodes][C][C] (in, out), and
 * the tensor-core copies are BF16 [nmodes][2C][2C].
 */
#ifndef WFS_FNO_H
#define WFS_FNO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* out[b][o] = act( sum_j W[o][j] in[b][j] + bias[o] + add[b][o] ), per site.
 * add, pre and copy may be NULL; pre receives the value before the activation,
 * copy a second copy of out (it may alias add). act: 0 none, 1 GELU (erf form).
 * Supported (cin, cout): cin, cout in {2, 4, 8, 16, 32, 64}. */
int wfs_fno_pointwise(const void* in, int32_t cin, const float* W, const float* bias, const void* add,
                      void* pre, void* out, void* copy, int32_t cout, int32_t B, int64_t n3, int32_t act,
                      void* stream);

/* Backward of wfs_fno_pointwise for one layer:
 *   gpre = (gout + gout2) * act'(pre)   (gout2 and pre may be NULL; act 0 ignores pre)
 *   gin  = W^T gpre                     (gin may be NULL)
 * gpre is stored (it feeds the weight gradient and the spectral branch). */
int wfs_fno_pointwise_backward(const void* gout, const void* gout2, const void* pre, int32_t act, const float* W,
                               void* gpre, void* gin, int32_t cin, int32_t cout, int32_t B, int64_t n3,
                               void* stream);

/* dW[o][j] = sum over samples and sites of g[o] x[j]; db[o] = sum of g[o].
 * Written to dWdb = [cout*cin weights][cout biases]. partials is scratch of
 * at least wfs_fno_wgrad_scratch(cin, cout) floats. */
int64_t wfs_fno_wgrad_scratch(int32_t cin, int32_t cout);
int wfs_fno_weight_grad(const void* g, int32_t cout, const void* x, int32_t cin, int32_t B, int64_t n3,
                        float* partials, float* dWdb, void* stream);

/* Unitary 3D DFT, in place, of nfields contiguous complex64 N^3 fields.
 * dir = -1 forward, +1 inverse. N must be a supported FFT length (wfs.h). */
int wfs_fno_fft3(void* data, int64_t nfields, int32_t N, int32_t dir, void* stream);

/* From the spectra of packed pairs (Y = F(h_2j + i h_2j+1)), the kept modes of
 * each real channel: Hm[mode][b][c] = F(h_c)(k_mode). */
int wfs_fno_gather(const void* spec, void* Hm, int32_t B, int32_t C, int32_t N, int32_t m, void* stream);

/* Inverse of the above: writes the whole spectra Y so that F^-1(Y) has real part
 * Re F^-1(Z_2j) and imaginary part Re F^-1(Z_2j+1), Z_c being Zm[.][.][c] placed on
 * the kept modes and 0 elsewhere (Y is cleared first). */
int wfs_fno_scatter(const void* Zm, void* spec, int32_t B, int32_t C, int32_t N, int32_t m, void* stream);

/* Tensor-core copies of the complex weights R: W = block form for the forward
 * product Z = H R, WT for the adjoint product G_H = G_Z R^H (both BF16). */
int wfs_fno_pack_weights(const float* R, void* W, void* WT, int32_t C, int32_t nmodes, void* stream);

/* Y[mode][b][:] = X[mode][b][:] . M(mode) on BF16 tensor cores with FP32
 * accumulation (mma.sync m16n8k16); Wsel is W (M = R) or WT (M = R^H).
 * C in {8, 16, 32} (2C must be a multiple of the MMA depth 16). */
int wfs_fno_mix(const void* X, const void* Wsel, void* Y, int32_t B, int32_t C, int32_t nmodes, void* stream);

/* dR[mode][i][o] = sum_b conj(H[mode][b][i]) G[mode][b][o]  (complex float32). */
int wfs_fno_spectral_weight_grad(const void* H, const void* G, float* dR, int32_t B, int32_t C, int32_t nmodes,
                                 void* stream);

/* Adam with decoupled weight decay over n float32 parameters. */
int wfs_fno_adam(float* p, const float* g, float* m1, float* m2, int64_t n, float lr, float beta1, float beta2,
                 float eps, float weight_decay, int32_t step, void* stream);

/* Per-sample relative squared error e_b = |pred_b - target_b|^2 / |target_b|^2
 * (per_sample floats each), loss = mean_b e_b, grad = grad_scale * d loss / d pred
 * (may be NULL). A grad_scale of per_sample trains on the per-element relative
 * error, whose gradients stay well above the optimiser's epsilon.
 * sample_err[B] and loss[1] are device floats. */
int wfs_fno_loss(const float* pred, const float* target, int64_t per_sample, int32_t B, float grad_scale,
                 float* sample_err, float* grad, float* loss, void* stream);

/* Per-sample |a_b|^2 and |a_b - c_b|^2 in FP64 (acceptance test of a jump). */
int wfs_fno_sample_norms(const void* a, const void* c, int64_t per_sample, int32_t B, double* a2, double* d2,
                         void* stream);

/* Network input from psi and V (both complex64 [B][n3]): x[b][0] = psi_b / s_b,
 * x[b][1] = V_b * vscale, with s_b = sqrt(a2_b / n3) the RMS of psi_b (a2 from
 * wfs_fno_sample_norms; NULL = no normalisation). */
int wfs_fno_make_input(const void* psi, const void* V, float vscale, const double* a2, void* x, int32_t B, int64_t n3,
                       void* stream);

/* a_b (complex64 [B][n3]) times s_b (invert = 0) or divided by s_b (invert = 1). */
int wfs_fno_scale_samples(void* a, const double* a2, int32_t invert, int32_t B, int64_t n3, void* stream);

/* ------------------------------------------------------------------------
 * Inference forward pass on the kept modes (csrc/fno_fast.cu). Same network and
 * parameters as above, for N = 64, width C = 32, m = 12 and projection width 64 only;
 * every product on BF16 tensor cores with FP32 accumulation and every intermediate
 * stored in BF16 (a jump's correction is about 1e-2 of psi, so this leaves the jump's
 * error unchanged). Arrays (32-bit words, each two BF16 values):
 *   H   [B][16][N^3]             channel pairs (2j, 2j+1)
 *   SY  [B][N x][24 ky][12 kz][32]  y- and z-spectra of each real channel on the kept
 *                                (ky, kz), (re, im)
 * One pass: lift; then per layer xmix and layer (the last layer: last). Each lift,
 * layer and last call handles one (sample, x) plane per CTA: the y and z DFTs of the
 * spectral branch, the pointwise layer and the activation stay on chip. All pointers
 * 16-byte aligned. */

/* h0 = W0 x + b0 with x = (psi / s_b, V * vscale) (4 real channels), s_b = sqrt(a2[b]
 * / N^3) (a2 NULL: s_b = 1), psi and V complex64 with sample strides psi_stride and
 * v_stride (complex values, even); W0p: BF16 [32][16] zero-padded. Writes H and the
 * kept y/z-spectra SY of h0. */
int wfs_fno_fast_lift(const void* psi, int64_t psi_stride, const void* V, int64_t v_stride, float vscale,
                      const double* a2, const void* W0p, const float* b0, void* h, void* sy, int32_t B,
                      void* stream);

/* h_out = GELU(W h_in + b + Re F^-1 Z) where SY holds the spectral branch Z (from
 * xmix); SY is then overwritten with the spectra of h_out. W: BF16 [32][32]. h_out
 * must not alias h_in. */
int wfs_fno_fast_layer(const void* h_in, void* sy, const void* W, const float* bias, void* h_out, int32_t B,
                       void* stream);

/* Last layer and both projections: out = prior + s_b (Wq2 GELU(Wq1 (W h_in + b +
 * Re F^-1 Z) + bq1) + bq2), prior and out complex64 [B][N^3], s_b as in the lift
 * (a2 NULL: 1). Wq1: BF16 [64][32]; Wq2p: BF16 [8][64], rows 2..7 zero. out_norm
 * (optional, B doubles) is incremented by sum |out_b|^2. */
int wfs_fno_fast_last(const void* h_in, const void* sy, const void* W, const float* bias, const void* Wq1,
                      const float* bq1, const void* Wq2p, const float* bq2, const void* prior, const double* a2,
                      void* out, double* out_norm, int32_t B, void* stream);

/* In place on SY: the unitary x DFT onto the 24 kept kx, Z = H R per kept mode (Wi from
 * wfs_fno_pack_mix_interleaved), and the inverse x DFT. */
int wfs_fno_fast_xmix(void* sy, const void* Wi, int32_t B, void* stream);

/* Limit of wfs_fno_fast_xmix's waits for its tensor-core commits, in seconds (default 1,
 * at most 60). A wait that gives up makes the CTA write NaN over its outputs (the jump then
 * fails its acceptance test), after the MMAs still in flight have drained. A limit of zero
 * makes every such wait give up at once: the test hook for that path. */
int wfs_fno_set_wait_limit(double seconds);

/* BF16 mixing weights with interleaved real and imaginary parts, in fragment order (see
 * wfs_fno_to_bf16): row 2o+s' of mode's block holds the coefficients of (Re, Im)[s] of
 * input channel i in (Re, Im)[s'] of output o, column k = 2i+s stored at the column d
 * with frag_src_col(d) = k. */
int wfs_fno_pack_mix_interleaved(const float* R, void* Wi, int32_t C, int32_t nmodes, void* stream);

/* dst (BF16 rows_pad x cols_pad) = src (float32 rows x cols), zero padded. With
 * frag_order (cols_pad a multiple of 16) the columns of each 16-column block are stored
 * in mma fragment order: column 4t+e holds source column 2t+e (e < 2) or 8+2t+e-2, so a
 * lane's B-fragment words for k = 2t, 2t+1 and 8+2t, 9+2t are adjacent (frag_src_col). */
int wfs_fno_to_bf16(const float* src, int32_t rows, int32_t cols, void* dst, int32_t rows_pad, int32_t cols_pad,
                    int32_t frag_order, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* WFS_FNO_H */
