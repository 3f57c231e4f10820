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

#ifdef __cplusplus
}
#endif
#endif
