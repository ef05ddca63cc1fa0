/*
 * oracle.c -- CPU restatement of the reference's raw-pixel -> PNG-scanline
 * arithmetic.  TEST INFRASTRUCTURE ONLY: this file is the checker that the
 * CUDA path is compared against.  It is never linked into, called by, or
 * used as a fallback for the product library; only the tests, the smoke
 * check and the CPU-baseline leg of the benchmark load it.
 *
 * Every function cites the reference file:line it restates (paths are
 * relative to the HeC-KriS/RAW2PNG-ConversionThruGPU project root).
 *
 * Floating point: compile with -O2 -ffp-contract=off so that no multiply-add
 * is fused (GCC on aarch64 contracts by default).  Division is IEEE FP32.
 *
 * Parity status:
 *   - 8-bit windowing (Q15 fast path + FP32 LUT fallback + their dispatch)
 *     is pinned against the reference's own C++ functions, compiled from its
 *     sources into oracle/_ref (see oracle/build_oracle.py) and exported as
 *     golden vectors under tests/golden/.
 *   - 16-bit windowing and the adaptive filter exist in the reference only as
 *     CUDA kernels (src/gpu_filter.cu); they are pinned against those kernels
 *     compiled from the reference sources and run on the GPU
 *     (tests/golden/gen_ref_gpu_golden.py writes the fixtures).
 */
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* Mirror of DicomPixelParams (include/dicom_params.h:6-21): same field
 * order, types and defaults. */
typedef struct orc_params {
    int   bits_allocated;
    int   bits_stored;
    int   high_bit;
    int   pixel_rep;
    int   apply_rescale;
    float rescale_slope;
    float rescale_intercept;
    int   apply_window;
    float window_center;
    float window_width;
} orc_params;

/* ------------------------------------------------------------------------
 * 16-bit-output windowing ("a2"): src/gpu_filter.cu:71-162
 * (dicom_preprocess_kernel), one sample at a time.
 *   raw  : bits_allocated==16 -> LE 16-bit sample; ==8 -> one byte
 *   out  : bits_allocated==16 -> 2 bytes big-endian; ==8 -> 1 byte
 * ---------------------------------------------------------------------- */
static uint32_t a2_sample(const uint8_t* in, size_t idx, const orc_params* p)
{
    const int out_maxval = (p->bits_allocated == 16) ? 65535 : 255;  /* :82 */
    float val;
    if (p->bits_allocated == 16) {
        uint16_t raw = (uint16_t)(in[idx * 2] | ((uint16_t)in[idx * 2 + 1] << 8)); /* :87-88 */
        int bit_shift = p->high_bit - p->bits_stored + 1;                           /* :93 */
        if (bit_shift > 0) raw = (uint16_t)(raw >> bit_shift);                      /* :94 */
        if (p->bits_stored < 16) {                                                  /* :97-100 */
            uint32_t mask = (1u << p->bits_stored) - 1u;
            raw = (uint16_t)(raw & (uint16_t)mask);
        }
        if (p->pixel_rep == 1) {                                                    /* :102-116 */
            int32_t sv;
            if (p->bits_stored == 16) {
                sv = (int32_t)(int16_t)raw;
            } else {
                int bits = p->bits_stored;
                int half = 1 << (bits - 1);
                sv = (int32_t)raw;
                if (sv >= half) sv -= (1 << bits);
            }
            if (p->apply_rescale) {
                float m = (float)sv * p->rescale_slope;
                val = m + p->rescale_intercept;
            } else {
                val = (float)sv;
            }
        } else {                                                                    /* :117-121 */
            val = (float)raw;
            if (p->apply_rescale) {
                float m = val * p->rescale_slope;
                val = m + p->rescale_intercept;
            }
        }
    } else {                                                                        /* :122-130 */
        if (p->pixel_rep == 1) val = (float)(int8_t)in[idx];
        else                   val = (float)in[idx];
        if (p->apply_rescale) {
            float m = val * p->rescale_slope;
            val = m + p->rescale_intercept;
        }
    }

    if (p->apply_window) {                                                          /* :136-151 */
        float wm1 = p->window_width - 1.0f;
        float cen = p->window_center;
        if (wm1 <= 0.0f) {
            val = (val >= cen) ? (float)out_maxval : 0.0f;
        } else {
            float half = wm1 * 0.5f;
            float lo = (cen - half) - 0.5f;
            float hi = (cen + half) - 0.5f;
            if (val <= lo)      val = 0.0f;
            else if (val > hi)  val = (float)out_maxval;
            else {
                float t = (val - cen) + 0.5f;
                float q = t / wm1;
                val = (q + 0.5f) * (float)out_maxval;
            }
        }
    }
    /* :153-154  clamp, then truncate toward zero.  fmaxf(0, fminf(max, v))
     * maps NaN to 0 (fminf/fmaxf return the non-NaN operand). */
    {
        float hi = (float)out_maxval;
        float v  = (val < hi) ? val : hi;
        if (val != val) v = hi;              /* fminf(hi, NaN) = hi */
        v = (v > 0.f) ? v : 0.f;
        return (uint32_t)v;
    }
}

void orc_window_a2(const uint8_t* in, size_t nsamples, const orc_params* p, uint8_t* out)
{
    for (size_t i = 0; i < nsamples; i++) {
        uint32_t ov = a2_sample(in, i, p);
        if (p->bits_allocated == 16) {            /* :156-161 big-endian store */
            out[i * 2]     = (uint8_t)(ov >> 8);
            out[i * 2 + 1] = (uint8_t)(ov & 0xFF);
        } else {
            out[i] = (uint8_t)ov;
        }
    }
}

/* ------------------------------------------------------------------------
 * 8-bit-output windowing, Q15 fast path ("a3"):
 * src/batch_processor.cpp:202-266 (try_apply_linear_window).
 * Returns 0 (and writes nothing) when the reference would decline.
 * Also exports the integer coefficients for the GPU kernel's parameter block.
 * ---------------------------------------------------------------------- */
int orc_q15_coeffs(const orc_params* p, int32_t* A_out, int32_t* B_out)
{
    const int shift = p->high_bit - p->bits_stored + 1;           /* :206-207 */
    if (shift != 0) return 0;
    float A_f, B_f;
    if (p->apply_window && p->window_width > 0.f) {               /* :214-220 */
        const float lo        = p->window_center - p->window_width * 0.5f;
        const float slope     = p->apply_rescale ? p->rescale_slope     : 1.f;
        const float intercept = p->apply_rescale ? p->rescale_intercept : 0.f;
        float t1 = slope * 255.f;
        A_f = t1 / p->window_width;
        float t2 = (intercept - lo) * 255.f;
        B_f = t2 / p->window_width;
    } else if (!p->apply_window) {                                /* :221-238 */
        const float slope     = p->apply_rescale ? p->rescale_slope     : 1.f;
        const float intercept = p->apply_rescale ? p->rescale_intercept : 0.f;
        const float range     = (float)(1u << p->bits_stored);
        if (p->pixel_rep == 1) {
            const float half = range * 0.5f;
            float t1 = slope * 255.f;
            A_f = t1 / range;
            float t2 = (intercept + half) * 255.f;
            B_f = t2 / range;
        } else {
            float r1 = range - 1.f;
            float t1 = slope * 255.f;
            A_f = t1 / r1;
            float t2 = intercept * 255.f;
            B_f = t2 / r1;
        }
    } else {
        return 0;                                                 /* :239-241 */
    }
    const float A_q15 = A_f * 32768.f;                            /* :243-245 */
    if (A_q15 < -32767.f || A_q15 > 32767.f) return 0;
    const int16_t A_fp = (int16_t)(int)A_q15;                     /* :247 */
    float bq;
    if (A_f >= 0.f) {                                             /* :248-251 */
        float bs = B_f * 32768.f;
        bq = (A_q15 == (float)(int)A_q15) ? bs : bs + 0.5f;
    } else {
        float bs = B_f * 32768.f;
        bq = bs - 0.5f;
    }
    *A_out = (int32_t)A_fp;
    *B_out = (int32_t)bq;
    return 1;
}

/* int32 arithmetic with two's-complement wrap, as the reference's int32
 * expression evaluates on the targets it runs on. */
static inline int32_t wrap_mad(int32_t x, int32_t a, int32_t b)
{
    uint32_t r = (uint32_t)x * (uint32_t)a + (uint32_t)b;
    return (int32_t)r;
}

int orc_window_q15(const uint8_t* src_le, size_t n, const orc_params* p, uint8_t* dst8)
{
    int32_t A, B;
    if (!orc_q15_coeffs(p, &A, &B)) return 0;
    for (size_t i = 0; i < n; i++) {                              /* :253-265 */
        uint16_t u16 = (uint16_t)(src_le[i * 2] | ((unsigned)src_le[i * 2 + 1] << 8));
        int32_t x = (p->pixel_rep == 1) ? (int32_t)(int16_t)u16 : (int32_t)u16;
        int32_t v = wrap_mad(x, A, B) >> 15;   /* arithmetic shift */
        dst8[i] = (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v);
    }
    return 1;
}

/* ------------------------------------------------------------------------
 * 8-bit-output FP32 LUT fallback ("a4"):
 * build_dicom16_lut  src/batch_processor.cpp:100-147
 * apply_dicom16_lut  src/batch_processor.cpp:157-185
 * ---------------------------------------------------------------------- */
void orc_build_lut(uint8_t* lut, const orc_params* p, int lut_size)
{
    const int mask = lut_size - 1;
    float norm_scale = 1.f, norm_offset = 0.f;
    if (!p->apply_window) {                                       /* :104-114 */
        if (p->pixel_rep == 1) {
            const float half  = (float)(lut_size >> 1);
            const float range = (float)lut_size;
            norm_scale  = 1.f / range;
            norm_offset = half / range;
        } else {
            norm_scale = 1.f / (float)(lut_size - 1);
        }
    }
    float lo = 0.f, inv_range = 1.f;
    if (p->apply_window) {                                        /* :116-121 */
        lo             = p->window_center - p->window_width * 0.5f;
        const float hi = p->window_center + p->window_width * 0.5f;
        inv_range      = (hi > lo) ? 1.f / (hi - lo) : 0.f;
    }
    for (int i = 0; i < lut_size; i++) {                          /* :124-146 */
        float val;
        if (p->pixel_rep == 1 && p->bits_stored < 16) {
            const int sign_bit = lut_size >> 1;
            int32_t s = i;
            if (s & sign_bit) s |= ~mask;
            val = (float)s;
        } else if (p->pixel_rep == 1) {
            val = (float)(int16_t)(uint16_t)(unsigned)i;
        } else {
            val = (float)(unsigned)i;
        }
        if (p->apply_rescale) {
            float m = val * p->rescale_slope;
            val = m + p->rescale_intercept;
        }
        float norm;
        if (p->apply_window) norm = (val - lo) * inv_range;
        else { float m = val * norm_scale; norm = m + norm_offset; }
        float s255 = norm * 255.f;
        const int v = (int)(s255 + 0.5f);
        lut[i] = (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v);
    }
}

void orc_apply_lut(const uint8_t* src_le, uint8_t* dst8, size_t n,
                   const uint8_t* lut, int shift, uint16_t mask16)
{
    for (size_t i = 0; i < n; i++) {                              /* :172-184 */
        const uint16_t raw = (uint16_t)((unsigned)src_le[i * 2] | ((unsigned)src_le[i * 2 + 1] << 8));
        dst8[i] = lut[(raw >> shift) & mask16];
    }
}

/* Dispatch of the 16-bit grayscale -> 8-bit conversion:
 * src/batch_processor.cpp:397-409 (Q15 first, LUT on decline; the LUT is
 * built with lut_size = 1 << bits_stored and shift/mask as in :306-318).
 * Returns 1 when the Q15 path ran, 2 when the LUT path ran. */
int orc_window8(const uint8_t* src_le, size_t n, const orc_params* p, uint8_t* dst8)
{
    if (orc_window_q15(src_le, n, p, dst8)) return 1;
    const int lut_size = 1 << p->bits_stored;
    uint8_t* lut = (uint8_t*)malloc((size_t)lut_size);
    if (!lut) return -1;
    orc_build_lut(lut, p, lut_size);
    orc_apply_lut(src_le, dst8, n, lut, p->high_bit - p->bits_stored + 1,
                  (uint16_t)(lut_size - 1));
    free(lut);
    return 2;
}

/* ------------------------------------------------------------------------
 * BMP export windowing: dicom16_row_to_gray8 (src/pipeline.cpp:1894-1932),
 * 16-bit LE grayscale DICOM -> 8-bit gray, with the normalisation constants
 * run_bmp_from_source passes it (:1953-1963).  Differs from the batch table
 * (orc_build_lut) only in dividing by (hi - lo) instead of multiplying by
 * its reciprocal.  Requires 0 <= high_bit - bits_stored + 1.
 * ---------------------------------------------------------------------- */
void orc_bmp_gray8(const uint8_t* src_le, size_t n, const orc_params* p, uint8_t* dst8)
{
    float norm_scale = 1.f, norm_offset = 0.f;
    if (!p->apply_window) {                                       /* :1953-1963 */
        if (p->pixel_rep == 1) {
            const float half  = (float)(1u << (p->bits_stored - 1));
            const float range = (float)(1u << p->bits_stored);
            norm_scale  = 1.f / range;
            norm_offset = half / range;
        } else {
            norm_scale = 1.f / (float)((1u << p->bits_stored) - 1u);
        }
    }
    const int shift = p->high_bit - p->bits_stored + 1;          /* :1899-1900 */
    const int mask  = (p->bits_stored < 32) ? ((1 << p->bits_stored) - 1) : -1;
    for (size_t i = 0; i < n; i++) {
        uint16_t raw = (uint16_t)((unsigned)src_le[i * 2] | ((unsigned)src_le[i * 2 + 1] << 8));
        raw = (uint16_t)((raw >> shift) & mask);
        float val;                                                /* :1906-1916 */
        if (p->pixel_rep == 1 && p->bits_stored < 16) {
            const int sign_bit = 1 << (p->bits_stored - 1);
            int32_t s = (int32_t)(uint32_t)raw;
            if (s & sign_bit) s |= ~((int32_t)mask);
            val = (float)s;
        } else if (p->pixel_rep == 1) {
            val = (float)(int16_t)raw;
        } else {
            val = (float)raw;
        }
        if (p->apply_rescale) {                                   /* :1918-1919 */
            float m = val * p->rescale_slope;
            val = m + p->rescale_intercept;
        }
        float norm;                                               /* :1921-1928 */
        if (p->apply_window) {
            const float h  = p->window_width * 0.5f;
            const float lo = p->window_center - h;
            const float hi = p->window_center + h;
            norm = (hi > lo) ? (val - lo) / (hi - lo) : 0.f;
        } else {
            float m = val * norm_scale;
            norm = m + norm_offset;
        }
        float s255 = norm * 255.f;                                /* :1930-1931 */
        const int v = (int)(s255 + 0.5f);
        dst8[i] = (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v);
    }
}

/* ------------------------------------------------------------------------
 * Adaptive PNG filter: src/gpu_filter.cu:183-309 (filter_select_kernel).
 *   img   : rows x rb windowed bytes (PNG byte order)
 *   prior : rb bytes seen as the row above row 0 (NULL = zeros)
 *   out   : rows x (rb + 1): [filter type][filtered bytes]
 * Score = sum over bytes of min(v, 256 - v) (:226); argmin with strict '<'
 * so the lowest type wins ties (:267-276); Average = (a+b)>>1 (:222);
 * Paeth prefers a, then b, then c (:212-216).
 * ---------------------------------------------------------------------- */
static inline uint8_t paeth(uint8_t a, uint8_t b, uint8_t c)
{
    const int pv = (int)a + (int)b - (int)c;
    const int pa = abs(pv - (int)a);
    const int pb = abs(pv - (int)b);
    const int pc = abs(pv - (int)c);
    return (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
}

static inline uint32_t cost(uint8_t v) { return v <= 128u ? (uint32_t)v : 256u - (uint32_t)v; }

void orc_filter_rows(const uint8_t* img, const uint8_t* prior, int rows, int rb, int bpp,
                     uint8_t* out)
{
    uint8_t* zeros = NULL;
    if (!prior) { zeros = (uint8_t*)calloc((size_t)rb + 1, 1); prior = zeros; }
    for (int r = 0; r < rows; r++) {
        const uint8_t* x = img + (size_t)r * rb;
        const uint8_t* up = (r > 0) ? img + (size_t)(r - 1) * rb : prior;
        uint32_t s[5] = {0, 0, 0, 0, 0};
        for (int i = 0; i < rb; i++) {
            const uint8_t a = (i >= bpp) ? x[i - bpp] : 0;
            const uint8_t b = up[i];
            const uint8_t c = (i >= bpp) ? up[i - bpp] : 0;
            s[0] += cost(x[i]);
            s[1] += cost((uint8_t)(x[i] - a));
            s[2] += cost((uint8_t)(x[i] - b));
            s[3] += cost((uint8_t)(x[i] - (uint8_t)(((unsigned)a + (unsigned)b) >> 1)));
            s[4] += cost((uint8_t)(x[i] - paeth(a, b, c)));
        }
        int best = 0; uint32_t bsc = s[0];
        for (int f = 1; f < 5; f++) if (s[f] < bsc) { bsc = s[f]; best = f; }
        uint8_t* o = out + (size_t)r * (rb + 1);
        o[0] = (uint8_t)best;
        for (int i = 0; i < rb; i++) {
            const uint8_t a = (i >= bpp) ? x[i - bpp] : 0;
            const uint8_t b = up[i];
            const uint8_t c = (i >= bpp) ? up[i - bpp] : 0;
            uint8_t pr;
            switch (best) {
                case 0: pr = 0; break;
                case 1: pr = a; break;
                case 2: pr = b; break;
                case 3: pr = (uint8_t)(((unsigned)a + (unsigned)b) >> 1); break;
                default: pr = paeth(a, b, c); break;
            }
            o[1 + i] = (uint8_t)(x[i] - pr);
        }
    }
    free(zeros);
}

/* Inverse of the five PNG filters (PNG specification, section 9): used to
 * decode produced PNGs back to pixel bytes.  Returns -1 on a bad type byte. */
int orc_unfilter(const uint8_t* filt, int rows, int rb, int bpp, uint8_t* out)
{
    for (int r = 0; r < rows; r++) {
        const uint8_t* f = filt + (size_t)r * (rb + 1);
        uint8_t* x = out + (size_t)r * rb;
        const uint8_t* up = (r > 0) ? out + (size_t)(r - 1) * rb : NULL;
        const int t = f[0];
        if (t > 4) return -1;
        for (int i = 0; i < rb; i++) {
            const uint8_t a = (i >= bpp) ? x[i - bpp] : 0;
            const uint8_t b = up ? up[i] : 0;
            const uint8_t c = (up && i >= bpp) ? up[i - bpp] : 0;
            uint8_t pr;
            switch (t) {
                case 0: pr = 0; break;
                case 1: pr = a; break;
                case 2: pr = b; break;
                case 3: pr = (uint8_t)(((unsigned)a + (unsigned)b) >> 1); break;
                default: pr = paeth(a, b, c); break;
            }
            x[i] = (uint8_t)(f[1 + i] + pr);
        }
    }
    return 0;
}
