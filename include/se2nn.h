/* se2nn.h -- C-ABI of libse2nn.so: the neural-operator surrogate of the
   se2wave solver, trained and evaluated on the GPU by hand-written sm_103a
   kernels (BF16 operands, FP32 accumulation; FP32 master weights and Adam).

   No counterpart in the reference (se2wave.c has no learned component).  The
   network maps the cell-wise material field plus a source channel to receiver
   traces.  Grid rows count down from the top surface (row 0), so the time axis
   of a receiver's trace lies along its column:

     input   x[b][y][x][cin]            BF16, channels last (cin a multiple of 16;
                                        the caller fills the used channels, the rest 0)
     lift    h = x W0 + b0               (1x1 convolution, cin -> width)
     layer l h = act(S_l(h) + h W_l + b_l),  act = GELU except for the last layer,
             S_l = spectral convolution: truncated real 2-D DFT keeping kx in
             [0, modes) and ky in [-modes, modes), per-mode complex width x width
             mixing, inverse DFT (1 / (nx ny) normalisation, Hermitian weights)
     decoder for receiver r (column rec_x[r]) and every row y, nsub = nout / ny:
             out[b][r][y][0:nsub] = GELU(h[b][y][rec_x[r]] W1 + c1) W2 + c2

   Parameters, as one FP32 vector in this order:
     W0 [cin][width], b0 [width];
     per layer: Wre [2 modes][modes][width][width], Wim (same), W [width][width], b [width];
     W1 [width][hidden], c1 [hidden], W2 [hidden][nsub], c2 [nsub].
   Mode (j, kx): ky = j for j < modes, ky = j - 2 modes (negative) otherwise.

   All pointers named *_dev are device memory; the others are host memory.
   Every call returns 0 or a negative code; se2nn_last_error gives the message. */
#ifndef SE2NN_H
#define SE2NN_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct se2nn_config {
  int ny, nx;        /* cell grid (128 x 128) */
  int cin;           /* input channels, multiple of 16 */
  int width;         /* channels of the hidden layers, multiple of 16 (64) */
  int modes;         /* retained modes per axis (16); 2 modes <= ny, modes <= nx / 2 */
  int layers;        /* Fourier layers (4) */
  int nrec;          /* receivers (16) */
  int nout;          /* outputs per receiver, a multiple of ny (2 components x 1024 samples) */
  int hidden;        /* decoder hidden width (128) */
  int max_batch;     /* largest batch of one call */
} se2nn_config;

typedef struct se2nn se2nn;

int  se2nn_create(const se2nn_config *cfg, unsigned long long seed, se2nn **out);
void se2nn_destroy(se2nn *h);
const char *se2nn_last_error(const se2nn *h);   /* NULL handle: last create failure */
int  se2nn_set_stream(se2nn *h, void *stream);
long se2nn_num_params(const se2nn *h);

/* FP32 parameters / gradients in the order above (host arrays of se2nn_num_params) */
int se2nn_get_params(se2nn *h, float *params);
int se2nn_set_params(se2nn *h, const float *params);
int se2nn_get_grads(se2nn *h, float *grads);

/* top-row cell index of each receiver (nrec ints in [0, nx)) */
int se2nn_set_receivers(se2nn *h, const int *rec_x);

/* out_dev[b][r][ny][nout / ny] (FP32) = network(x_dev[b]) for b < batch */
int se2nn_forward(se2nn *h, const void *x_dev, int batch, float *out_dev);

/* Forward and backward of the mean-squared error against target_dev[b][r][nout]
   (FP32): loss = mean((out - target)^2) over batch*nrec*nout values.  The
   gradients of the loss replace the handle's gradient buffer; *loss (host)
   receives the loss, out_dev (optional) the network output. */
int se2nn_loss_grad(se2nn *h, const void *x_dev, int batch, const float *target_dev, double *loss, float *out_dev);

/* One Adam step (bias-corrected, decoupled weight decay) with the current
   gradients; the step counter is kept by the handle. */
int se2nn_adam_step(se2nn *h, float lr, float beta1, float beta2, float eps, float weight_decay);

/* Input assembly from a resident data set: for b < batch, sample s = idx_dev[b]:
   materials_dev[s][y][x][3] holds (vp, vs, rho) per cell (FP32 m/s, m/s, kg/m^3)
   with row y counted up from the bottom, src_dev[s] the source position in cells
   (x, y up from the bottom).  Network row yn is material row ny - 1 - yn:
   channels 0..2 = (vp - 5000) / 1500, (vs - 2800) / 800, (rho - 2500) / 500,
   channel 3 = exp(-|cell centre - source|^2 / (2 sigma^2)) (source at row
   coordinate ny - y), channels 4, 5 = cell-centre coordinates in [-1, 1] (x, yn),
   the rest 0.  x_dev[b][yn][x][cin] (BF16). */
int se2nn_build_inputs(se2nn *h, const void *materials_dev, const float *src_dev, const int *idx_dev, int batch,
                       float sigma_cells, void *x_dev);

/* Gather target rows: out_dev[b] = targets_dev[idx_dev[b]] (nrec*nout FP32 values each). */
int se2nn_gather_targets(se2nn *h, const float *targets_dev, const int *idx_dev, int batch, float *out_dev);

/* Strided-batched BF16 GEMM of the network's kernel (exposed for tests):
   C[b] = alpha op(A[b]) op(B[b]) + beta C[b], op(A) M x K, op(B) K x N, C FP32
   row-major with leading dimension ldc; transA/transB as in the kernel. */
int se2nn_gemm(const void *A_dev, const void *B_dev, float *C_dev, int M, int N, int K, int batch, long lda, long ldb,
               long ldc, long sA, long sB, long sC, int transA, int transB, float alpha, float beta, void *stream);

/* Tensor-core path of the row GEMMs (no counterpart in the reference).  Row GEMMs --
   one batch, k-contiguous A, at least 128 rows, K and N multiples of 16 up to 128: the
   lift, the 1x1 convolutions, the decoder and their data gradients -- can run on the
   5th-generation tensor cores (tcgen05.mma, accumulators in tensor memory), the others
   run on the mma.sync kernel.  mode 0: every GEMM on mma.sync; 1 (default): the row
   GEMMs on tcgen05 except those with N <= 64 and 32 < K <= 64 (the 1x1 convolutions,
   where mma.sync measured faster); 2: every row GEMM on tcgen05.  Process-wide.  se2nn_tensor_path_info: out[0] = tcgen05 GEMM launches,
   out[1] = mma.sync GEMM launches, out[2] = 1 if a tcgen05 GEMM's bounded wait ever
   expired. */
int se2nn_set_tensor_path(int mode);
int se2nn_tensor_path_info(long out[3]);

#ifdef __cplusplus
}
#endif
#endif
