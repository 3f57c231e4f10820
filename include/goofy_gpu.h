/*
 * goofy_gpu.h -- C ABI of the GB300 (sm_103a) Goofy BC1 / ETC1s block encoder.
 *
 * Plain pointers and sizes only; `stream` arguments are cudaStream_t passed as
 * void* (NULL = the legacy default stream).  Every function returns a status
 * code (GOOFY_OK or a negative GOOFY_ERR_*).
 *
 * Output format and bits are those of the reference goofy::compressDXT1 /
 * goofy::compressETC1 (GoofyTC/goofy_tc.h:10-13, defined at :1497-1557):
 * (width/4)*(height/4) blocks of 8 bytes, row-major, no destination pitch.
 */
#ifndef GOOFY_GPU_H
#define GOOFY_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define GOOFY_OK 0
#define GOOFY_ERR_WIDTH (-1)     /* same code as the reference (goofy_tc.h:1500-1503) */
#define GOOFY_ERR_HEIGHT (-2)    /* same code as the reference (goofy_tc.h:1505-1508) */
#define GOOFY_ERR_INVALID (-3)   /* null pointer, stride < 4*width, bad codec, ... */
#define GOOFY_ERR_ALIGNMENT (-4) /* device source not 4-byte aligned / dst not 8-byte aligned */
#define GOOFY_ERR_CUDA (-5)      /* a CUDA runtime call failed; see goofy_gpu_last_error() */
#define GOOFY_ERR_NOMEM (-6)     /* device or pinned host allocation failed */
#define GOOFY_ERR_TIMEOUT (-7)   /* a bounded wait expired */
#define GOOFY_ERR_BUSY (-8)      /* queue / admission budget exhausted */
#define GOOFY_ERR_NO_DEVICE (-9) /* no usable CUDA device */
#define GOOFY_ERR_TOO_LARGE (-10) /* request exceeds a fixed capacity */

#define GOOFY_CODEC_BC1 0   /* DXT1 / BC1, goofySimdEncode<GOOFY_DXT1> */
#define GOOFY_CODEC_ETC1S 1 /* ETC1s, goofySimdEncode<GOOFY_ETC1> */
#define GOOFY_CODEC_BOTH 2  /* both from one read of the image: goofy_gpu_compress_both_*, and the
                             * tile of that pass in goofy_gpu_{get,set}_tile only */

/* ---- library -------------------------------------------------------------- */

/* Select the device the host-pointer entry points use (default: device 0) and
 * create its streams.  Optional: the first host call initialises lazily.
 * No reference counterpart (the reference is a pure CPU function). */
int goofy_gpu_init(int device);

/* Release every resource the library holds (streams, staging, arenas). */
void goofy_gpu_shutdown(void);

/* Human-readable text for a status code. */
const char* goofy_gpu_status_string(int status);

/* Text of the last CUDA error the library saw on this thread ("" if none). */
const char* goofy_gpu_last_error(void);

/* ---- device pointers (asynchronous on `stream`) ---------------------------- */

/* Device-pointer variant of goofy::compressDXT1 (goofy_tc.h:1497-1526).
 * src: device RGBA8, `stride` bytes per row (4-byte aligned; 16-byte aligned
 * src and stride take the vector-load path).  dst: device, 8-byte aligned,
 * (width/4)*(height/4)*8 bytes.  width % 4 == 0 (not % 16: blocks are
 * independent), height % 4 == 0.  Enqueues one kernel on `stream`; no sync.
 * The kernel is launched with programmatic stream serialization: after one of
 * this library's kernels its CTAs may be scheduled while that kernel drains,
 * but they touch no global memory before it has completed, so stream order
 * holds for every buffer (after any other kernel or copy it starts when that
 * one completes).  The decoders and the mip generator launch the same way. */
int goofy_gpu_compress_bc1_device(void* dst, const void* src, uint32_t width, uint32_t height,
                                  uint32_t stride, void* stream);

/* Device-pointer variant of goofy::compressETC1 (goofy_tc.h:1528-1557). */
int goofy_gpu_compress_etc1s_device(void* dst, const void* src, uint32_t width, uint32_t height,
                                    uint32_t stride, void* stream);

/* Either codec (GOOFY_CODEC_BC1 or GOOFY_CODEC_ETC1S). */
int goofy_gpu_compress_device(int codec, void* dst, const void* src, uint32_t width, uint32_t height,
                              uint32_t stride, void* stream);

/* ---- host pointers (synchronous, drop-in semantics) ------------------------ */

/* Host-memory counterpart of goofy::compressDXT1 (goofy_tc.h:1497-1526): same
 * arguments and output, returns when `dst` holds the result.  Pinned or
 * pageable buffers of any alignment; width % 4 == 0, height % 4 == 0.  When
 * the GPU can address both buffers (pinned memory, or any host memory where
 * it walks the host page tables, as on Grace-Blackwell) and they are word
 * aligned, one kernel reads the rows and writes the blocks over the host
 * link; otherwise the image is streamed through device memory in bands (copy
 * in / encode / copy out overlapped on two streams).  See
 * goofy_gpu_set_host_path.  Thread-safe (calls are serialised). */
int goofy_gpu_compress_bc1_host(uint8_t* dst, const uint8_t* src, uint32_t width, uint32_t height,
                                uint32_t stride);

/* Host-memory counterpart of goofy::compressETC1 (goofy_tc.h:1528-1557). */
int goofy_gpu_compress_etc1s_host(uint8_t* dst, const uint8_t* src, uint32_t width, uint32_t height,
                                  uint32_t stride);

/* Either codec (GOOFY_CODEC_BC1 or GOOFY_CODEC_ETC1S). */
int goofy_gpu_compress_host(int codec, uint8_t* dst, const uint8_t* src, uint32_t width, uint32_t height,
                            uint32_t stride);

/* ---- both codecs from one read of the image -------------------------------- */

/* The BC1 blocks of goofy::compressDXT1 into `dst_bc1` and the ETC1s blocks
 * of goofy::compressETC1 into `dst_etc1s` ((width/4)(height/4)*8 bytes each),
 * bit-identical to the two single-codec calls, from one pass over `src`: the
 * image is read once (4 B/px instead of the two calls' 8; 1 B/px written
 * either way) and the per-block work both encoders share (channel extents, brightness range,
 * per-pixel luma sums) is done once.  No reference counterpart: the reference
 * harness calls the two encoders one after the other on every image
 * (Src/main.cpp:925-929).  Same rules as the single-codec calls; outputs
 * that overlap are refused (GOOFY_ERR_INVALID).  Device form: async on `stream`, with the tile of
 * GOOFY_CODEC_BOTH.  Host form: synchronous, pinned or pageable buffers. */
int goofy_gpu_compress_both_device(void* dst_bc1, void* dst_etc1s, const void* src, uint32_t width,
                                   uint32_t height, uint32_t stride, void* stream);
int goofy_gpu_compress_both_host(uint8_t* dst_bc1, uint8_t* dst_etc1s, const uint8_t* src, uint32_t width,
                                 uint32_t height, uint32_t stride);

/* How the host-pointer entry points move data (process-wide setting):
 * AUTO (default): DIRECT when both buffers are GPU-accessible -- pinned
 * memory, or any host memory where the GPU walks the host page tables
 * (Grace-Blackwell NVLink-C2C) -- and suitably aligned, else STAGED.
 * STAGED: copy bands into device buffers, encode there, copy back.
 * DIRECT: one kernel reads the caller's rows and writes its blocks over the
 * host link; GOOFY_ERR_INVALID if the buffers do not allow it. */
#define GOOFY_HOST_PATH_AUTO 0
#define GOOFY_HOST_PATH_STAGED 1
#define GOOFY_HOST_PATH_DIRECT 2
int goofy_gpu_set_host_path(int path);
int goofy_gpu_get_host_path(void);

/* ---- pinned host memory (for callers that want the fast host path) -------- */
void* goofy_gpu_host_alloc(size_t bytes);
void goofy_gpu_host_free(void* p);

/* ---- tile shape (launch configuration of the image kernel) ---------------- */
typedef struct goofy_gpu_tile {
    uint32_t threads_per_cta;   /* 128, 256, 512 */
    uint32_t blocks_per_thread; /* 4x4 blocks a thread encodes per segment: 1, 2, 4 (1, 2 if persistent) */
    uint32_t persistent;        /* 0: one segment per warp; 1: resident grid, loop with prefetch;
                                 * 2: resident grid, one producer warp streams tiles into a
                                 *    shared-memory ring with bulk async copies (1, 2 blocks per
                                 *    thread; 16-byte aligned sources, others run shape 0) */
} goofy_gpu_tile;

/* Get / set the tile the image kernels launch with, per codec
 * (GOOFY_CODEC_BOTH: the two-codec pass; 1 or 2 blocks a thread, and mode 1
 * runs as mode 0 there).  Compiled default for every codec: 512 threads,
 * 2 blocks a thread, mode 2. */
int goofy_gpu_get_tile(int codec, goofy_gpu_tile* tile);
int goofy_gpu_set_tile(int codec, const goofy_gpu_tile* tile);

/* Autotuner: times every tile shape on the caller's device image (`src`,
 * `dst` as for goofy_gpu_compress_device, on the current device) with CUDA
 * events -- after two warm-up launches, three rounds of `reps` launches back to
 * back between two events, the median round's mean kept -- installs the
 * fastest as the codec's tile and returns it with that mean launch time in
 * microseconds.  Synchronous.  No reference counterpart.  GOOFY_CODEC_BOTH
 * tunes the two-codec pass: `dst` then holds both outputs back to back
 * (2 * (width/4)(height/4)*8 bytes, the BC1 blocks first). */
int goofy_gpu_autotune(int codec, void* dst, const void* src, uint32_t width, uint32_t height, uint32_t stride,
                       uint32_t reps, goofy_gpu_tile* best, float* best_us);

/* Autotuner for callers that encode every image with both codecs, one call
 * after the other (as the reference harness calls goofy::compressDXT1 and
 * goofy::compressETC1 on each image): ranks each codec's tiles alone as
 * goofy_gpu_autotune does, then times the alternating BC1 / ETC1s launches on
 * the image for the pairs of each codec's finalists -- its three fastest
 * tiles and its three fastest bulk-copy tiles (mode 2); a shape that is
 * fastest alone can leave a gap where the other codec's launch takes over
 * the SMs -- and installs the fastest pair.  best_us: the mean time of one
 * BC1 + ETC1s pair.  Both outputs (dst_bc1, dst_etc1s) must not overlap.
 * Synchronous.  No reference counterpart. */
int goofy_gpu_autotune_pair(void* dst_bc1, void* dst_etc1s, const void* src, uint32_t width, uint32_t height,
                            uint32_t stride, uint32_t reps, goofy_gpu_tile* best_bc1, goofy_gpu_tile* best_etc1s,
                            float* best_us);

/* ---- tile cache: tuned tiles kept per GPU model --------------------------- */
/* No reference counterpart (the reference has no launch shape to tune).  The
 * fastest tile differs between boxes of the same GPU model, so
 * goofy_gpu_autotune records its pick in a text file keyed by GPU name and SM
 * count, and goofy_gpu_init -- or, without it, a process's first encode call
 * (the drop-in goofy::compressDXT1 / compressETC1 included) -- installs the
 * recorded tile of every codec whose tile was not set explicitly
 * (goofy_gpu_set_tile, goofy_gpu_autotune).  Without an entry the compiled
 * defaults stay.  Tiles are process-wide, not per device: with several GPU
 * models in one process the last one loaded wins.
 * File: the path given to goofy_gpu_set_tile_cache_path, else
 * $GOOFY_TILE_CACHE ("" disables the cache), else
 * $XDG_CACHE_HOME/goofy_gb300/tiles.txt, else $HOME/.cache/goofy_gb300/tiles.txt.
 * One entry per line, "v1|<GPU name>|<SM count>|<bc1|etc1s|both>|<threads>|
 * <blocks a thread>|<mode>|<microseconds>"; lines that do not parse, name a
 * tile the kernels cannot run or belong to another GPU model are ignored.  A
 * write replaces the file atomically (temporary file + rename); a cache that
 * cannot be written leaves the autotuner's result in effect for the process. */
int goofy_gpu_set_tile_cache_path(const char* path); /* NULL: back to the environment / default */
/* The path in use; copies at most size-1 bytes and a NUL into buf (may be
 * NULL) and returns the full length. */
size_t goofy_gpu_get_tile_cache_path(char* buf, size_t size);
/* The GPU name and SM count that key `device`'s entries. */
int goofy_gpu_device_key(int device, char* name, size_t size, uint32_t* sm_count);
/* Record / look up one entry directly (path NULL: the path in use).  Need no
 * GPU.  lookup returns GOOFY_ERR_INVALID when there is no valid entry. */
int goofy_gpu_tile_cache_store(const char* path, const char* gpu_name, uint32_t sm_count, int codec,
                               const goofy_gpu_tile* tile, float us);
int goofy_gpu_tile_cache_lookup(const char* path, const char* gpu_name, uint32_t sm_count, int codec,
                                goofy_gpu_tile* tile);
/* Installs `device`'s cached tiles now (codecs not set explicitly); returns
 * how many were installed, or a negative status. */
int goofy_gpu_load_tile_cache(int device);
/* Restores the compiled default tiles and forgets which were set explicitly;
 * the cache is read again by the next goofy_gpu_init or encode call. */
int goofy_gpu_reset_tiles(void);

/* Waits of the bulk-copy pipeline (tile mode 2) that gave up after their
 * time limit on the current device (each ends its kernel early instead of
 * hanging); `reset` != 0 zeroes the count.  0 in a healthy run.  Synchronous. */
int goofy_gpu_pipeline_timeouts(uint32_t* count, int reset);

/* Self-test of the bounded waits on the current device.  One thread of a
 * one-warp kernel waits on an mbarrier that nothing completes (no copy, no
 * arrival); its wait gives up after the limit every pipeline wait has (1 s),
 * raises its CTA's abort flag and counts one time-out in a counter of this
 * call's own.  GOOFY_OK when exactly that happened and the kernel returned
 * (the context stays usable), GOOFY_ERR_CUDA otherwise.  `elapsed_ms`, if not
 * NULL, receives the call's wall time.  Synchronous, about one second. */
int goofy_gpu_selftest_bounded_wait(uint32_t* elapsed_ms);

/* ---- decoding and encode quality -------------------------------------------- */

/* Decode (width/4)*(height/4) blocks (device) into RGBA8 rows (device,
 * `rgba` and `rgba_stride` 16-byte aligned), as the reference harness's
 * decoders do (Src/decoder.cpp:933-971): BC1 in both endpoint orders; ETC1
 * individual and differential modes with flip, alpha 255.  ETC1 differential
 * blocks whose second colour leaves 0..31 (ETC2 modes) decode to zeros and
 * are added to *d_unsupported (device uint64).  Asynchronous. */
int goofy_gpu_decode_device(int codec, void* rgba, uint32_t rgba_stride, const void* blocks, uint32_t width,
                            uint32_t height, uint64_t* d_unsupported, void* stream);

/* Adds to d_sums[0..5] (device uint64) the integer core of the reference's
 * getMsePsnr (Src/main.cpp:403-469) between `src` (RGBA8, 4-byte aligned
 * rows) and its decoded `blocks`: [0..3] per-byte sums of squared
 * differences, [4] the unsupported-block count, [5] the sum of squared
 * luminosity differences in hundredths, (21 d2 + 72 d1 + 7 d0)^2 with dk the
 * difference of byte k -- the harness's 0.21 R + 0.72 G + 0.07 B of a pixel
 * read as a little-endian u32, exact in integers.  Asynchronous. */
int goofy_gpu_block_error_device(int codec, const void* blocks, const void* src, uint32_t width, uint32_t height,
                                 uint32_t stride, uint64_t* d_sums, void* stream);

/* Synchronous convenience: RGB PSNR (peak 768, as the reference reports it)
 * of `blocks` against `src`, both on the current device; sums_out (may be
 * NULL) receives accumulators [0..4] above. */
int goofy_gpu_psnr_rgb(int codec, const void* blocks, const void* src, uint32_t width, uint32_t height,
                       uint32_t stride, double* psnr_rgb, uint64_t* sums_out);

/* The harness's MsePsnr record (Src/main.cpp:366-384), same field meaning and
 * channel naming (a pixel read as a little-endian u32: r = byte 2, b = byte 0). */
typedef struct goofy_gpu_quality {
    double mse_r, mse_g, mse_b, mse_a, mse_max, mse_rgb, mse_y;
    double psnr_r, psnr_g, psnr_b, psnr_a, psnr_min, psnr_rgb, psnr_y;
    uint64_t unsupported_blocks;
} goofy_gpu_quality;

/* Synchronous: getMsePsnr(src, decode(blocks)) computed on the current device.
 * Every MSE except mse_y equals the harness's double result exactly (its sums
 * are exact integers); mse_y differs only by the harness's own rounding of
 * its 0.21 / 0.72 / 0.07 products (relative < 1e-10 on its test photographs,
 * far below the 5 decimals it prints). */
int goofy_gpu_mse_psnr(int codec, const void* blocks, const void* src, uint32_t width, uint32_t height,
                       uint32_t stride, goofy_gpu_quality* out);

/* ---- mip chains on the device -------------------------------------------------- */

/* One level of a mip chain on the device. */
typedef struct goofy_gpu_level {
    void* data;
    uint32_t width, height, stride;
} goofy_gpu_level;

/* Levels of the chain of a width x height texture (each axis halves,
 * clamped at 4, down to 4x4); 0 unless both sizes are powers of two >= 4. */
uint32_t goofy_gpu_mip_count(uint32_t width, uint32_t height);

/* Device bytes goofy_gpu_generate_mips needs for levels 1.. (256-byte rows). */
size_t goofy_gpu_mip_arena_bytes(uint32_t width, uint32_t height);

/* Build levels 1.. of the chain of `src` (device RGBA8) into `arena`
 * (device, 256-byte aligned) with a 2x2 box filter with rounding,
 * (a+b+c+d+2)>>2 per channel (an axis already at 4 is copied), and describe
 * all levels (levels[0] = src) for goofy_gpu_batch_encode.  No reference
 * counterpart (the reference encodes levels the caller made).  Async. */
int goofy_gpu_generate_mips(const void* src, uint32_t width, uint32_t height, uint32_t stride, void* arena,
                            size_t arena_bytes, goofy_gpu_level* levels, uint32_t max_levels, uint32_t* nlevels,
                            void* stream);

/* ---- PNG ingest (host) ------------------------------------------------------------
 * Replaces the harness's image loader, loadPngAsRgba8 (Src/main.cpp:258-342:
 * lodepng::decode to 8-bit RGBA, alpha then forced to 255).  Every colour type
 * and bit depth and both interlace methods; CRCs and Adler-32 verified; 16-bit
 * samples keep their high byte, 1/2/4-bit grey scales by 255/(2^depth-1),
 * tRNS gives alpha 0 to the key colour (lodepng's conversion rules).
 * GOOFY_ERR_INVALID for a malformed file (text in goofy_gpu_last_error()). */

/* Width and height from the IHDR chunk. */
int goofy_gpu_png_info(const void* png, size_t png_bytes, uint32_t* width, uint32_t* height);

/* Decode into RGBA8 rows of `stride` bytes (host memory, `rgba_bytes` long);
 * `opaque` != 0 sets every alpha to 255 as the harness does.  width / height
 * (may be NULL) receive the image size even when the buffer is too small
 * (GOOFY_ERR_TOO_LARGE). */
int goofy_gpu_png_decode(const void* png, size_t png_bytes, void* rgba, size_t rgba_bytes, uint32_t stride,
                         int opaque, uint32_t* width, uint32_t* height);

/* ---- containers ---------------------------------------------------------------- */

/* Bytes of the container of `levels` levels (host blocks): DDS for BC1, KTX
 * 1.1 for ETC1s.  0 for invalid arguments. */
size_t goofy_gpu_container_size(int codec, const uint32_t* widths, const uint32_t* heights, uint32_t levels);

/* Write header + levels into `out`: DDS ("DXT1" FourCC) for BC1, KTX 1.1
 * (GL_ETC1_RGB8_OES) for ETC1s.  With one level the bytes equal the
 * reference harness's saveDds / saveKtx output (Src/main.cpp:154-220);
 * several levels form a mip chain (level 0 first). */
int goofy_gpu_write_container(int codec, const uint8_t* const* level_blocks, const uint32_t* widths,
                              const uint32_t* heights, uint32_t levels, uint8_t* out, size_t out_size);

/* The harness's TGA image (saveTga, Src/main.cpp:222-255): an 18-byte header
 * (type 2, 32 bits per pixel, top-left origin) and BGRA pixels, from RGBA8
 * rows.  goofy_gpu_tga_size is 0 for sizes TGA cannot hold (above 65535). */
size_t goofy_gpu_tga_size(uint32_t width, uint32_t height);
int goofy_gpu_write_tga(const uint8_t* rgba, uint32_t stride, uint32_t width, uint32_t height, uint8_t* out,
                        size_t out_size);

/* ---- batches: many device images of uneven sizes in one launch ----------- */

/* One image of a batch (a texture or one of its mip levels).  src / dst and
 * the size rules are those of goofy_gpu_compress_device; codec per image. */
typedef struct goofy_gpu_image {
    const void* src;
    void* dst;
    uint32_t width, height, stride;
    int32_t codec; /* GOOFY_CODEC_* */
} goofy_gpu_image;

typedef struct goofy_gpu_batch goofy_gpu_batch;

typedef struct goofy_gpu_batch_tile {
    uint32_t threads_per_cta;   /* 128, 256, 512 (compute threads; the pipeline adds a producer warp) */
    uint32_t blocks_per_thread; /* 1 or 2 */
    uint32_t unit_blocks;       /* 4x4 blocks per work unit, a multiple of 32 * blocks_per_thread;
                                 * threads_per_cta * blocks_per_thread with pipeline = 1 */
    uint32_t pipeline;          /* 0: warps pull work units and load their rows themselves;
                                 * 1: per CTA a producer warp pulls units and bulk-copies their rows
                                 *    into a shared-memory ring, compute warps encode from there */
} goofy_gpu_batch_tile;

/* A batch object for up to `max_images` images per call on `device`; owns its
 * descriptor tables, work counters, stream and graphs.  No reference
 * counterpart (the reference encodes one image per call). */
int goofy_gpu_batch_create(goofy_gpu_batch** batch, uint32_t max_images, int device);
void goofy_gpu_batch_destroy(goofy_gpu_batch* batch);

/* Encode `count` images in one persistent launch: warps pull work units
 * (runs of unit_blocks blocks of one image) from a device work counter, or
 * with a pipeline tile each CTA's producer warp stages its units' rows in
 * shared memory.  Enqueued on `stream` (one descriptor upload and the
 * kernel, a CUDA graph replay for a repeated batch shape; with a pipeline
 * tile and at most 64 images, the descriptors are the kernel's parameter and
 * nothing is uploaded): ordered after the work already queued there, and
 * later work there waits for it.  Each image's output equals
 * goofy_gpu_compress_device on that image alone. */
int goofy_gpu_batch_encode(goofy_gpu_batch* batch, const goofy_gpu_image* images, uint32_t count, void* stream);

/* CUDA-graph replay of same-shaped batches (default on). */
int goofy_gpu_batch_set_graphs(goofy_gpu_batch* batch, int enable);
int goofy_gpu_batch_get_tile(goofy_gpu_batch* batch, goofy_gpu_batch_tile* tile);
int goofy_gpu_batch_set_tile(goofy_gpu_batch* batch, const goofy_gpu_batch_tile* tile);

/* Time every batch tile on this set of images, keep the fastest for this
 * batch object: per tile two warm-up launches, then three rounds of `reps`
 * launches back to back between two CUDA events, the median round's mean
 * per launch.  Writes the images' outputs as a side effect.  Synchronous. */
int goofy_gpu_batch_autotune(goofy_gpu_batch* batch, const goofy_gpu_image* images, uint32_t count, uint32_t reps,
                             goofy_gpu_batch_tile* best, float* best_us);

/* ---- serving: continuous batching of host-memory requests ----------------- */

#define GOOFY_SERVER_STAGED 0 /* requests copied into a device arena, encoded there, copied back */
#define GOOFY_SERVER_DIRECT 1 /* the batch kernel reads / writes the requests' host buffers itself */

/* How the server learns that a launch has finished. */
#define GOOFY_SERVER_COMPLETION_CALLBACK 0 /* a host function enqueued after the launch (cudaLaunchHostFunc),
                                            * run by the CUDA driver's thread; it also holds back the next
                                            * launch's work on that stream until it has run */
#define GOOFY_SERVER_COMPLETION_EVENT 1    /* a thread of the server waits on each launch's last event in
                                            * turn (a blocking-sync event: the thread sleeps, no spinning);
                                            * nothing is added to the streams */

typedef struct goofy_gpu_server goofy_gpu_server;

typedef struct goofy_gpu_server_config {
    int32_t device;
    int32_t mode;                  /* GOOFY_SERVER_STAGED or GOOFY_SERVER_DIRECT */
    uint64_t device_budget_bytes;  /* admission budget: arena size (staged) or bytes in flight (direct) */
    uint32_t max_batch_images;     /* requests folded into one launch */
    uint32_t max_inflight_batches; /* launches on the GPU at once */
    uint32_t max_requests;         /* unreleased tickets at once */
    uint32_t quality;              /* 1: measure every request's RGB PSNR on the GPU (harness's getMsePsnr) */
    uint32_t completion;           /* GOOFY_SERVER_COMPLETION_CALLBACK (default) or _EVENT */
} goofy_gpu_server_config;

/* One encode request on host memory (pinned buffers are copied by DMA / read
 * by the GPU directly; direct mode needs GPU-accessible buffers). */
typedef struct goofy_gpu_request {
    const uint8_t* src;
    uint8_t* dst;
    uint32_t width, height, stride;
    int32_t codec;
} goofy_gpu_request;

typedef struct goofy_gpu_request_times {
    int64_t submit_ns, admit_ns, launch_ns, done_ns; /* goofy_gpu_now_ns() clock */
    double psnr_rgb; /* with config.quality: RGB PSNR of the blocks as the harness reports it (peak 768), else 0 */
} goofy_gpu_request_times;

typedef struct goofy_gpu_server_stats {
    uint64_t launches, requests_done, pixels_done, max_batch, waiting, inflight_bytes;
    /* Launch timing since the previous goofy_gpu_server_get_stats call (read
     * and reset by each call), to tell where a late request lost its time.
     * Maxima over the launches: the scheduler thread's time in the CUDA calls
     * that enqueue one launch (copies, kernels, callback), the GPU time of
     * one launch's batch kernel (CUDA events around it), and the time from
     * the start of a launch's enqueue to its completion callback. */
    uint64_t max_enqueue_ns, max_kernel_ns, max_launch_ns;
    /* The parts of the launch that took max_launch_ns: its enqueue time, the
     * GPU time from its first operation to its last (events on the copy /
     * compute streams; it includes waits behind earlier launches' work once
     * its first operation has run) and its kernel time.  What max_launch_ns
     * has beyond the enqueue and the GPU span was spent before the GPU
     * reached the launch or in delivering its completion callback. */
    uint64_t slowest_enqueue_ns, slowest_gpu_span_ns, slowest_kernel_ns;
} goofy_gpu_server_stats;

/* Defaults: device 0, staged, 16 GiB budget, 1024 requests per launch, 4
 * launches in flight, 2^20 tickets.  No reference counterpart (the reference
 * is a synchronous per-image function). */
void goofy_gpu_server_default_config(goofy_gpu_server_config* cfg);

/* Start a server (allocates its arena, launch slots and streams once, and a
 * scheduler thread).  Requests that arrive while others run are admitted as
 * budget frees up and join the next launch of the persistent batch kernel. */
int goofy_gpu_server_create(goofy_gpu_server** server, const goofy_gpu_server_config* cfg);

/* Stop after finishing everything submitted; release all resources. */
void goofy_gpu_server_destroy(goofy_gpu_server* server);

/* Queue one request; never blocks on the GPU.  GOOFY_ERR_TOO_LARGE if the
 * request alone exceeds the budget, GOOFY_ERR_BUSY if max_requests tickets
 * are unreleased.  Output equals goofy_gpu_compress_host on the same request. */
int goofy_gpu_server_submit(goofy_gpu_server* server, const goofy_gpu_request* req, uint64_t* ticket);

/* Wait up to timeout_ms for a ticket; on completion returns its status, fills
 * `times` (may be NULL) and releases the ticket.  GOOFY_ERR_TIMEOUT leaves the
 * ticket pending. */
int goofy_gpu_server_wait(goofy_gpu_server* server, uint64_t ticket, uint32_t timeout_ms,
                          goofy_gpu_request_times* times);

int goofy_gpu_server_get_stats(goofy_gpu_server* server, goofy_gpu_server_stats* stats);

/* Monotonic clock of the request timestamps, in nanoseconds. */
int64_t goofy_gpu_now_ns(void);

/* Open-loop load replay: submits reqs[i] at start + arrival_ns[i] while a
 * second thread waits on the tickets; latency_ns[i] = completion - scheduled
 * arrival (-1 if it failed); wall_ns = start to last completion; times (may be
 * NULL) receives each request's submit / admit / launch / completion stamps. */
int goofy_gpu_server_replay(goofy_gpu_server* server, const goofy_gpu_request* reqs, const int64_t* arrival_ns,
                            uint32_t n, int64_t* latency_ns, int64_t* wall_ns, goofy_gpu_request_times* times);

/* The same replay through the plain loop: one request at a time, each a
 * host->device copy, one image-kernel launch and a device->host copy. */
int goofy_gpu_plain_replay(int device, const goofy_gpu_request* reqs, const int64_t* arrival_ns, uint32_t n,
                           int64_t* latency_ns, int64_t* wall_ns);

/* ---- batch encoding without any allocation ---------------------------------- */

/* Largest image count goofy_gpu_batch_encode_noalloc takes per call. */
#define GOOFY_NOALLOC_MAX_IMAGES 256

/* Encodes a batch like goofy_gpu_batch_encode (same images, same output) but
 * allocates nothing, for callers that may not call cudaMalloc / cudaFree or
 * any allocating routine while they encode -- e.g. a texture-streaming thread
 * inside a renderer's frame budget, where the CUDA allocator can stall the
 * device, or an engine whose own allocator owns all GPU memory.  No
 * counterpart in the reference.
 * The work counter and descriptor tables live in one fixed file-scope device
 * array of the library (13,568 bytes, held on every GPU that loads the library
 * until the process exits), so a call takes at most GOOFY_NOALLOC_MAX_IMAGES
 * images; more returns GOOFY_ERR_TOO_LARGE, a NULL `images` with count > 0
 * GOOFY_ERR_INVALID, and an invalid image its status -- all before anything
 * is launched.  The caller's images (device src / dst) are the inputs and
 * outputs; they must be on the calling thread's current device, whose copy of
 * the array the call uses.  The first call in a context (a device's primary
 * context, again after cudaDeviceReset) looks up the array's device address
 * with cudaGetSymbolAddress; make that first call before any stream capture.
 * All calls share the array: calls whose GPU work overlaps (e.g. on two
 * unordered streams) race; issue them on one stream or order them.
 * Asynchronous on `stream`: two launches, a small kernel that takes the
 * call's tables as its parameter and writes them into the array, then the
 * batch kernel; no host memory is read after the call returns. */
int goofy_gpu_batch_encode_noalloc(const goofy_gpu_image* images, uint32_t count, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GOOFY_GPU_H */
