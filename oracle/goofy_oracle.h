/*
 * goofy_oracle.h -- CPU oracle for the Goofy BC1/ETC1s block encoder.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * encoder (GoofyTC/goofy_tc.h, goofy::compressDXT1 / goofy::compressETC1) used
 * as the parity checker by tests/, by __graft_entry__.smoke() and by the CPU
 * baseline legs of bench.py.  The product (goofy_gb300/) never links, loads
 * or calls it.
 *
 * Parity pinning: the restatement is checked bit-for-bit against the
 * reference compiled from its own header (oracle/ref_shim.cpp, built by
 * oracle/build.py into oracle/_ref/ where the reference sources exist) and
 * against the golden vectors under tests/golden/ that the reference produced.
 */
#ifndef GOOFY_ORACLE_H
#define GOOFY_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_BC1 = 0, ORACLE_ETC1S = 1 };

/* Encode one 4x4 block whose top-left pixel is at `p` (RGBA8, `stride` bytes
 * between rows) into 8 output bytes. */
void oracle_encode_block(int codec, const uint8_t* p, size_t stride, uint8_t out[8]);

/* Same contract as goofy::compressDXT1/compressETC1 (goofy_tc.h:1497-1557):
 * returns -1 when width % 16 != 0, -2 when height % 4 != 0, else 0.  Output is
 * (width/4)*(height/4) blocks of 8 bytes, row-major, no destination pitch. */
int oracle_compress(int codec, uint8_t* result, const uint8_t* input,
                    unsigned width, unsigned height, unsigned stride);

/* Generalisation used for narrow mip levels: width % 4 == 0 is enough
 * (-1 otherwise); blocks are independent, so this equals the reference run on
 * rows padded to a multiple of 16 pixels with the padding blocks dropped. */
int oracle_compress_any(int codec, uint8_t* result, const uint8_t* input,
                        unsigned width, unsigned height, unsigned stride);

/* oracle_compress_any striped by block rows over `threads` POSIX threads
 * (threads <= 0: one per online CPU).  Returns the thread count used, or a
 * negative error as above. */
int oracle_compress_mt(int codec, uint8_t* result, const uint8_t* input,
                       unsigned width, unsigned height, unsigned stride, int threads);

/* ---- decode and error (the reference's quality check) ---------------------
 * Decode one 8-byte block into 16 RGBA8 pixels (row-major, 64 bytes).
 * BC1: both endpoint orders (4-colour and 3-colour + transparent black), as
 * Src/decoder.cpp:799-871 (DecompressColour) + :933-943 (decodeBlockDXT1).
 * ETC1: individual and differential modes with flip, alpha 255, as
 * Src/decoder.cpp:388-678 (decompressBlockDiffFlipC) + :958-971.  A
 * differential block whose second colour leaves 0..31 is an ETC2 mode
 * (decoder.cpp:740-760); those decode to zeros and return -1, else 0. */
int oracle_decode_block(int codec, const uint8_t blk[8], uint8_t out[64]);

/* Decode a whole image (width, height multiples of 4) into RGBA8 rows of
 * `stride` bytes.  Returns the number of unsupported ETC1 blocks. */
long oracle_decode_image(int codec, const uint8_t* blocks, unsigned width, unsigned height, uint8_t* rgba,
                         unsigned stride);

/* Per-channel sums of squared differences between two RGBA8 images (bytes 0..3
 * of each pixel), the integer core of getMsePsnr (Src/main.cpp:403-469). */
void oracle_sq_error(const uint8_t* a, unsigned a_stride, const uint8_t* b, unsigned b_stride, unsigned width,
                     unsigned height, uint64_t sums[4]);

/* RGB PSNR exactly as getMsePsnr / getPSNR compute psnrRGB (peak 768,
 * Src/main.cpp:386-395, :455, :466) from the sums above. */
double oracle_psnr_rgb(const uint64_t sums[4], unsigned width, unsigned height);

/* The harness's full getMsePsnr (Src/main.cpp:403-469) in its own double
 * arithmetic, pixel order and channel naming (a pixel read as a little-endian
 * u32: R = byte 2, B = byte 0).  out = mseR, mseG, mseB, mseA, mseMax, mseRGB,
 * mseY, psnrR, psnrG, psnrB, psnrA, psnrMin, psnrRGB, psnrY. */
void oracle_mse_psnr(const uint8_t* a, unsigned a_stride, const uint8_t* b, unsigned b_stride, unsigned width,
                     unsigned height, double out[14]);

#ifdef __cplusplus
}
#endif
#endif
