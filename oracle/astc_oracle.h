/*
 * astc_oracle.h -- CPU oracle for the ASTC block encoder.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle that the CUDA
 * encoder is compared against; it is never linked into, loaded by or called
 * from the product library (libastc_gb300.so) or the CLI.  Only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark use it.
 *
 * It restates the reference compute shader (ASTC_Encode.hlsl,
 * ASTC_IntegerSequenceEncoding.hlsl, ASTC_Table.hlsl of niepp/astc_encoder)
 * on the CPU:
 *   - oracle_encode_fp32  : FP32, the shader's operation order, one fixed
 *                           arithmetic model (see astc_oracle.cpp header);
 *   - oracle_encode_fp64  : the same steps evaluated in double (quality twin);
 *   - oracle_decode       : integer-only ASTC LDR decoder written from the
 *                           ASTC specification (Khronos Data Format Spec,
 *                           "ASTC" chapter), UNORM8 output.
 */
#ifndef ASTC_ORACLE_H
#define ASTC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_opts {
    int block_dim;   /* 4 or 6                                              */
    int has_alpha;   /* HAS_ALPHA    (ASTC_Encode.hlsl:13-15)               */
    int is_normal;   /* IS_NORMALMAP (ASTC_Encode.hlsl:17-19, 575-578)      */
    int srgb;        /* texels are sRGB-decoded before the fit (main.cpp:38)*/
    int border;      /* 0 = zero outside the texture (D3D11 Load rule),
                        1 = clamp to the edge texel                         */
    int axis;        /* 0 = principal_component_analysis (the shader's
                        call, ASTC_Encode.hlsl:514), 1 = the shader's
                        alternative max_accumulation_pixel_direction
                        (170-227, commented out at 515), 2 = both, keeping
                        the fit whose fixed-mode block decodes with the
                        smaller squared error (the PCA on ties)             */
    int quality;     /* 0 = the shader's fixed mode (518-522); 1 = search:
                        the fixed-mode block plus every single-partition
                        4x4-grid weight range QUANT_3..QUANT_32 with the
                        largest endpoint range that fits, keeping the
                        candidate whose decode has the least squared error
                        against the texels rounded to bytes in the fit
                        space (the choose_best_quantmethod the shader
                        sketches at 524-526); 2 = the same search from the
                        better of the two fits (both axes tried, the one
                        whose fixed-mode block has the smaller error kept,
                        the PCA on ties; axis is then ignored) plus
                        dual-plane candidates (one channel on plane 2,
                        chosen by the residual of the covariance without
                        it; every legal weight range scored); 3 = 2 plus
                        two-partition candidates (one partition pattern,
                        matched to the split of the kept fit, each
                        partition fitted on its own, every legal weight
                        range scored); 4 = 3 plus three-partition
                        candidates (the four pattern classes that best
                        match an integer three-colour labelling)          */
} oracle_opts;

/* Encode a tightly packed RGBA8 image (row 0 first) into 16-byte blocks in
 * row-major block order.  threads <= 0 uses every OpenMP thread.
 * Returns 0 on success, negative on bad arguments. */
int oracle_encode_fp32(const uint8_t* rgba, int width, int height,
                       const oracle_opts* opts, uint8_t* out_blocks, int threads);
int oracle_encode_fp64(const uint8_t* rgba, int width, int height,
                       const oracle_opts* opts, uint8_t* out_blocks, int threads);

/* Per-block FP32 encode exposing the symbolic intermediate results:
 * ep[8] = quantised endpoints r0 r1 g0 g1 b0 b1 a0 a1,
 * qw[16] = quantised (unscrambled) weights.  texels: N*4 floats (0..255). */
int oracle_encode_block_fp32(const float* texels, int block_dim, int has_alpha,
                             uint32_t ep[8], uint32_t qw[16], uint8_t out[16]);

/* Integer stages only: assemble a block from symbolic endpoints and weights
 * (weight quant method QUANT_6 when has_alpha, QUANT_12 otherwise). */
/* The intermediate values of the FP32 fixed-mode pipeline for one block, for
 * the tests that explain each block where the oracle and the reference's own
 * output differ (which rounding or comparison decided it, and by how much). */
typedef struct oracle_trace {
    float start_w;              /* alpha of the power iteration's start vector:
                                   0 in the shader (ASTC_Encode.hlsl:96); a
                                   trace may seed it to model rounding noise  */
    float mean[4], cov[16];     /* principal_component_analysis 139-162       */
    int early_exit;             /* eigen_vector iteration (1..8) that returned
                                   early on length(v) < 1e-5, else 0 (93-106) */
    float min_len;              /* the smallest length(v) the test saw        */
    float axis[4];              /* eigen_vector's result                      */
    float tmin, tmax;           /* find_min_max projections (108-118)         */
    float e0_fit[4], e1_fit[4]; /* clamped endpoints before the swap (120-121) */
    float s0, s1;               /* rounded RGB sums compared for the swap     */
    int swapped;                /* s0 > s1 (125-129)                          */
    float e0[4], e1[4];         /* final endpoints (alpha forced without -alpha)*/
    float wlen;                 /* length(e1 - e0) in calculate_normal_weights */
    float wproj[16];            /* dot(k, texel - e0) before scaling (316-356) */
    float minw, maxw, inv;      /* the scaling (358-366)                      */
    float wR[16];               /* scaled weight x range, before round (256-260)*/
    uint32_t ep[8], qw[16];     /* quantised endpoints r0 r1 g0 g1 ..., weights */
    uint8_t block[16];          /* the assembled block                        */
} oracle_trace;
int oracle_trace_block_fp32(const float* texels, int block_dim, int has_alpha, float start_w,
                            oracle_trace* tr);
/* The first of n_seeds start-vector alpha seeds under which the FP32
 * fixed-mode pipeline assembles exactly `target`; -1 if none does. */
int oracle_find_seed(const float* texels, int block_dim, int has_alpha, const uint8_t target[16],
                     const float* seeds, int n_seeds);

int oracle_assemble_symbolic(const uint32_t ep[8], const uint32_t qw[16],
                             int has_alpha, uint8_t out[16]);

/* Bounded integer sequence encoding of `count` values in quant method
 * `quant` (0..20, QUANT_2..QUANT_256).  Writes LSB-first into out[16]. */
int oracle_ise_encode(int quant, int count, const uint32_t* values, uint8_t out[16]);
/* Inverse of the above (spec decode).  Returns 0 on success. */
int oracle_ise_decode(int quant, int count, const uint8_t in[16], int bit_offset,
                      uint32_t* values);
int oracle_ise_bits(int quant, int count);

/* Tables generated from the spec definitions (never copied). */
void oracle_table_trits(int out[243]);     /* integer_from_trits        */
void oracle_table_quints(int out[125]);    /* integer_from_quints       */
void oracle_table_btq(int out[63]);        /* bits_trits_quints_table   */
void oracle_table_scramble(int out[384]);  /* scramble_table, 12 x 32   */
void oracle_srgb_lut(float out[256]);      /* sRGB code -> linear * 255 */

/* Integer-only ASTC LDR decoder (UNORM8 out, tightly packed RGBA8).
 * Error blocks decode to magenta (255,0,255,255).  Returns the number of
 * error blocks, or negative on bad arguments. */
int oracle_decode(const uint8_t* blocks, int width, int height,
                  int block_w, int block_h, int srgb, uint8_t* out_rgba);
/* Decode one block (used by the property tests). */
int oracle_decode_block(const uint8_t blk[16], int block_w, int block_h, int srgb,
                        uint8_t* out_rgba);
/* Spec unquantisation of one weight (to 0..64) / one colour value (0..255). */
int oracle_unquant_weight(int quant, int value);
int oracle_unquant_color(int quant, int value);

/* The 2x2 texel taps and weights of grid point g (0..15) of the 4x4 weight
 * grid of a 6x6 block (idx_grids / wt_grids, ASTC_Encode.hlsl:268-304). */
void oracle_grid_taps(int g, int idx[4], float wt[4]);

/* Algorithmic FP32 operation count of one block, counted by running the
 * FP32 pipeline with counting arithmetic (FMA counted as 2). */
double oracle_flops_per_block(int block_dim, int has_alpha, int is_normal);

/* Search mode introspection.  Endpoint quant method the ASTC decoder derives
 * for a single-partition 4x4 weight grid of weight quant method `wq` and
 * `nvals` endpoint values (6 = CEM 8, 8 = CEM 12), or -1 if the mode is
 * invalid. */
int oracle_endpoint_quant(int wq, int nvals);
/* The three-partition pattern classes of a block size (4 or 6): the smallest
 * partition index of each distinct split of the block into three non-empty
 * sets, in index order, with the texels of its partitions 1 and 2 (bit
 * y * dim + x).  Writes up to cap entries; returns the class count. */
int oracle_three_classes(int dim, int* seeds, uint64_t* m1, uint64_t* m2, int cap);
/* Encode one block (texels: N*4 floats, 0..255, the fit space) in search
 * mode with FP32 arithmetic (axis 2: from the better of both fits, with
 * dual-plane candidates; partitions 1: two-partition candidates as well, 2:
 * two- and three-partition candidates).  *chosen_wq = weight quant method of
 * the block kept (-1 when the fixed-mode block was kept, 100 + wq for a
 * two-partition block, 200 + 16 * plane-2 channel + wq for a dual-plane
 * block, 300 + 16 * class rank + wq for a three-partition block), *err = the
 * squared error of its decode against the texels rounded to bytes,
 * *err_fixed = the fixed-mode block's. */
int oracle_search_block_fp32(const float* texels, int block_dim, int has_alpha, int srgb, int axis,
                             int partitions, uint8_t out[16], int* chosen_wq, uint32_t* err,
                             uint32_t* err_fixed);

#ifdef __cplusplus
}
#endif
#endif
