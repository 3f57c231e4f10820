"""Command-line front end of the GPU encoder.

  python -m goofy_gb300.tool run [--data DIR] [--images a,b,...] [--iterations N] [--out DIR]
      The reference harness's per-image run (Src/main.cpp:826-987, runTest)
      with this library as the encoder: each PNG is loaded as the harness
      loads it, encoded to ETC1 and DXT1 through the drop-in entry points
      (host buffers, best of N wall-clock runs, as runTestETC1 / runTestDXT1
      time them, :646-664), measured with the harness's getMsePsnr record
      (on the GPU) and printed as the harness's result rows
      (Image;Encoder;Format;NumberOfPixels;time (us);MP/s;mse...;psnr...;delta...),
      deltas against its RGB565 downsample baseline row.  With --out it
      writes the files the harness writes: DDS / KTX blocks, the decoded
      images (decoded on the GPU) and the original and baseline images as
      TGA.

  python -m goofy_gb300.tool autotune [--size N] [--cache PATH]
      Tunes the image-kernel tiles on this GPU (both codecs together, then
      the two-codec pass) on a synthetic NxN scene and records them in the
      tile cache, which later processes' first calls install.

  python -m goofy_gb300.tool encode IN.png OUT.dds|OUT.ktx [--codec bc1|etc1s] [--mips] [--both]
      One PNG to a DDS (BC1) or KTX (ETC1s) file, optionally with a full mip
      chain generated on the GPU (power-of-two sizes) and all levels encoded
      in one batch launch.  --both writes OUT with the .dds and with the .ktx
      extension from one pass per level (goofy_gpu_compress_both_device).
"""
import argparse
import ctypes
import glob
import os
import sys
import time

import numpy as np

import goofy_gb300 as g

HEADER = ("Image;Encoder;Format;NumberOfPixels;time (us);MP/s;mseR;mseG;mseB;mseMax;mseRGB;mseY;psnrR (db);"
          "psnrG (db);psnrB (db);psnrMin (db);psnrRGB (db);psnrY (db);deltaMin (db);deltaRGB (db);deltaY (db)")
ENCODER = "gb300_goofy"


def psnr_text(p):
    """psnrToString, Src/main.cpp:472-482."""
    return "+inf" if p > 999999.0 else "%3.5f" % p


def baseline_rgb565(img, w, h):
    """The harness's quality baseline, generateDownsamlpedRgb565Test
    (Src/main.cpp:501-557): 2x2 box average with rounding, quantised to
    5/6/6 bits and widened again by bit replication, alpha 255.  Channel
    names follow the harness (a pixel read as a little-endian u32: r = byte 2,
    b = byte 0)."""
    px = img.reshape(h // 2, 2, w // 2, 2, 4)[..., :3].astype(np.uint32)
    s = (px.sum(axis=(1, 3)) + 2) >> 2
    b, gch, r = s[..., 0], s[..., 1], s[..., 2]
    r, gch, b = r >> 3, gch >> 2, b >> 2
    r = (r << 3) | ((r >> 2) & 7)
    gch = (gch << 2) | ((gch >> 4) & 3)
    b = (b << 2) | ((b >> 2) & 7)
    q = np.stack([b, gch, r, np.full_like(r, 255)], axis=-1).astype(np.uint8)
    return np.repeat(np.repeat(q, 2, axis=0), 2, axis=1).reshape(h, 4 * w)


def mse_psnr_images(a, b, w, h):
    """getMsePsnr (Src/main.cpp:403-469) of two host images in exact integers
    (luminosity in hundredths, as the GPU measurement sums it)."""
    d = a.reshape(h, w, 4).astype(np.int64) - b.reshape(h, w, 4).astype(np.int64)
    sq = (d * d).reshape(-1, 4).sum(axis=0)
    y = 21 * d[..., 2] + 72 * d[..., 1] + 7 * d[..., 0]
    n = float(np.uint32(w * h))
    q = {"mse_r": sq[2] / n, "mse_g": sq[1] / n, "mse_b": sq[0] / n, "mse_a": sq[3] / n,
         "mse_rgb": float(sq[0] + sq[1] + sq[2]) / n, "mse_y": float((y * y).sum()) / 10000.0 / n}
    q = {k: float(v) for k, v in q.items()}
    q["mse_max"] = max(q["mse_r"], q["mse_g"], q["mse_b"], q["mse_a"])

    def psnr(m, peak=255.0):
        return sys.float_info.max if m < 0.0000001 else 10.0 * np.log10((peak * peak) / m)

    for c in "rgba":
        q["psnr_" + c] = psnr(q["mse_" + c])
    q["psnr_min"] = min(q["psnr_r"], q["psnr_g"], q["psnr_b"], q["psnr_a"])
    q["psnr_rgb"] = psnr(q["mse_rgb"], 768.0)
    q["psnr_y"] = psnr(q["mse_y"])
    return q


def result_row(image, encoder, fmt, pixels, time_us, q, base):
    """One line as runTest prints it (Src/main.cpp:950-974)."""
    mps = (pixels / (time_us / 1e6)) / 1e6 if time_us > 0 else 0.0
    fields = ["%3.5f" % q[k] for k in ("mse_r", "mse_g", "mse_b", "mse_max", "mse_rgb", "mse_y")]
    fields += [psnr_text(q[k]) for k in ("psnr_r", "psnr_g", "psnr_b", "psnr_min", "psnr_rgb", "psnr_y")]
    deltas = ["%3.5f" % (q[k] - base[k]) for k in ("psnr_min", "psnr_rgb", "psnr_y")]
    return ";".join([image, encoder, fmt, "%3.0f" % pixels, "%3.0f" % time_us, "%3.5f" % mps] + fields + deltas)


def write(folder, name, data):
    with open(os.path.join(folder, name), "wb") as f:
        f.write(data)


def run_image(path, iterations, out_dir, torch):
    """Result rows for one photograph (baseline, ETC1, DXT1), or None when
    the harness would refuse it (width % 16, height % 4)."""
    name = os.path.splitext(os.path.basename(path))[0]
    img, w, h = g.read_png(path)
    if w % 16 or h % 4:
        print("%s: %dx%d refused (width must be a multiple of 16, height of 4)" % (name, w, h), file=sys.stderr)
        return None
    base_img = baseline_rgb565(img, w, h)
    base = mse_psnr_images(img, base_img, w, h)
    rows = [result_row(name, "Baseline (Downsample x2)", "RGB565", w * h, 0, base, base)]
    d_src = torch.from_numpy(img.reshape(-1)).cuda()
    if out_dir:
        write(out_dir, name + "_original.tga", g.tga(img, w, h))
        write(out_dir, name + "_baseline.tga", g.tga(base_img, w, h))
    for codec, fmt, fn, kind, ext in ((g.CODEC_ETC1S, "ETC1", g.compressETC1, "etc1", "ktx"),
                                      (g.CODEC_BC1, "DXT1", g.compressDXT1, "dxt1", "dds")):
        out = np.zeros(g.out_size(w, h), np.uint8)
        best = float("inf")
        for _ in range(iterations):
            t0 = time.perf_counter()
            rc = fn(out, img, w, h, 4 * w)
            best = min(best, (time.perf_counter() - t0) * 1e6)
            if rc != 0:
                raise RuntimeError("%s: encode failed %d %s" % (name, rc, g.last_error()))
        d_blocks = torch.from_numpy(out).cuda()
        q = g.mse_psnr(codec, d_blocks, d_src, w, h, 4 * w)
        rows.append(result_row(name, ENCODER, fmt, w * h, best, q, base))
        if out_dir:
            stem = "%s_%s_%s" % (name, ENCODER, kind)
            write(out_dir, stem + "." + ext, g.container(codec, [(out, w, h)]))
            rgba = torch.empty(4 * w * h, dtype=torch.uint8, device="cuda")
            bad = torch.zeros(1, dtype=torch.int64, device="cuda")
            assert g.decode_device(codec, rgba, 4 * w, d_blocks, w, h, bad) == g.OK, g.last_error()
            torch.cuda.synchronize()
            write(out_dir, stem + "_decompressed.tga", g.tga(rgba.cpu().numpy().reshape(h, 4 * w), w, h))
    return rows


def cmd_run(args):
    import torch

    if g.init(0) != g.OK:
        raise SystemExit("no usable GPU: " + g.last_error())
    if args.out:
        os.makedirs(args.out, exist_ok=True)
    names = args.images.split(",") if args.images else None
    paths = [os.path.join(args.data, n + ".png") for n in names] if names else sorted(
        glob.glob(os.path.join(args.data, "*.png")))
    print(HEADER)
    for p in paths:
        rows = run_image(p, args.iterations, args.out, torch)
        for r in rows or ():
            print(r, flush=True)
    return 0


def cmd_encode(args):
    import torch

    codec = {"bc1": g.CODEC_BC1, "etc1s": g.CODEC_ETC1S}[args.codec or (
        "etc1s" if args.output.lower().endswith(".ktx") else "bc1")]
    img, w, h = g.read_png(args.input)
    if w % 4 or h % 4:
        raise SystemExit("%s: %dx%d is not a whole number of 4x4 blocks" % (args.input, w, h))
    if g.init(0) != g.OK:
        raise SystemExit("no usable GPU: " + g.last_error())
    d_src = torch.from_numpy(img.reshape(-1)).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    levels = [(d_src.data_ptr(), w, h, 4 * w)]
    arena = None
    if args.mips:
        nbytes = g.lib().goofy_gpu_mip_arena_bytes(w, h)
        if not nbytes and g.lib().goofy_gpu_mip_count(w, h) == 0:
            raise SystemExit("--mips needs power-of-two sizes >= 4")
        arena = torch.empty(nbytes + 256, dtype=torch.uint8, device="cuda")
        base = arena.data_ptr() + (-arena.data_ptr()) % 256
        levels = g.generate_mips(d_src, w, h, 4 * w, base, nbytes, stream)
    if args.both:
        return _encode_both(args, levels, stream, torch)
    outs = [torch.empty(g.out_size(lw, lh), dtype=torch.uint8, device="cuda") for _, lw, lh, _ in levels]
    batch = g.Batch(len(levels))
    try:
        rc = batch.encode([(p, o.data_ptr(), lw, lh, s, codec) for (p, lw, lh, s), o in zip(levels, outs)], stream)
        if rc != g.OK:
            raise SystemExit("encode failed: %s %s" % (g.status_string(rc), g.last_error()))
        torch.cuda.synchronize()
    finally:
        batch.close()
    data = g.container(codec, [(o.cpu().numpy(), lw, lh) for o, (_, lw, lh, _) in zip(outs, levels)])
    with open(args.output, "wb") as f:
        f.write(data)
    print("%s: %dx%d, %d level(s), %s, %d bytes" % (args.output, w, h, len(levels), args.codec or
                                                   ("etc1s" if codec else "bc1"), len(data)))
    return 0


def _encode_both(args, levels, stream, torch):
    """Every level through the two-codec pass: the BC1 blocks to OUT.dds and
    the ETC1s blocks to OUT.ktx, each level read once."""
    outs = []
    for p, lw, lh, s in levels:
        n = g.out_size(lw, lh)
        o = torch.empty(2 * n, dtype=torch.uint8, device="cuda")
        rc = g.compress_both_device(o.data_ptr(), o.data_ptr() + n, p, lw, lh, s, stream)
        if rc != g.OK:
            raise SystemExit("encode failed: %s %s" % (g.status_string(rc), g.last_error()))
        outs.append((o, n, lw, lh))
    torch.cuda.synchronize()
    stem = os.path.splitext(args.output)[0]
    for codec, ext, half in ((g.CODEC_BC1, ".dds", 0), (g.CODEC_ETC1S, ".ktx", 1)):
        host = [(o[half * n:(half + 1) * n].cpu().numpy(), lw, lh) for o, n, lw, lh in outs]
        data = g.container(codec, host)
        with open(stem + ext, "wb") as f:
            f.write(data)
        print("%s: %d level(s), %s, %d bytes" % (stem + ext, len(outs), "bc1" if codec == g.CODEC_BC1 else "etc1s",
                                                len(data)))
    return 0


def cmd_autotune(args):
    """Tune the tiles on a synthetic scene of the given size and record them
    in the tile cache (goofy_gpu_autotune_pair for BC1 and ETC1s, then
    goofy_gpu_autotune for the two-codec pass)."""
    import torch

    from . import workloads

    if args.cache is not None:
        g.set_tile_cache_path(args.cache)
    if not g.tile_cache_path():
        raise SystemExit("the tile cache is disabled (GOOFY_TILE_CACHE is empty); give --cache PATH")
    assert g.init(args.device) == g.OK, g.last_error()
    torch.cuda.set_device(args.device)
    w = h = args.size
    img = workloads.scene(w, h, 1, max(1, w // 256), max(8, w * h // 32768), threads=0)
    src = torch.from_numpy(img.reshape(-1)).cuda()
    n = g.out_size(w, h)
    out = torch.empty(2 * n, dtype=torch.uint8, device="cuda")
    t_bc1, t_etc1s, us = g.autotune_pair(out.data_ptr(), out.data_ptr() + n, src.data_ptr(), w, h, 4 * w,
                                         reps=args.reps)
    t_both, us_both = g.autotune(g.CODEC_BOTH, out.data_ptr(), src.data_ptr(), w, h, 4 * w, reps=args.reps)
    name, sms = g.device_key(args.device)
    print("%s (%d SMs), %dx%d scene: bc1 %s + etc1s %s, %.2f us a pair; both-codec pass %s, %.2f us" %
          (name, sms, w, h, t_bc1, t_etc1s, us, t_both, us_both))
    print("recorded in", g.tile_cache_path())
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m goofy_gb300.tool", description=__doc__.split("\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    r = sub.add_parser("run", help="the harness's per-image result rows with the GPU encoder")
    r.add_argument("--data", default="test-data", help="folder of PNG files (the harness's test-data/)")
    r.add_argument("--images", help="comma-separated image names (default: every PNG in --data)")
    r.add_argument("--iterations", type=int, default=128, help="timed runs per encode; the best is kept")
    r.add_argument("--out", help="folder for the DDS / KTX files")
    e = sub.add_parser("encode", help="PNG to DDS (BC1) or KTX (ETC1s)")
    e.add_argument("input")
    e.add_argument("output")
    e.add_argument("--codec", choices=("bc1", "etc1s"))
    e.add_argument("--mips", action="store_true", help="add a GPU-generated mip chain")
    e.add_argument("--both", action="store_true", help="write OUT.dds and OUT.ktx from one pass over each level")
    t = sub.add_parser("autotune", help="tune the kernel tiles for this GPU and record them in the tile cache")
    t.add_argument("--size", type=int, default=8192, help="side of the synthetic scene to tune on")
    t.add_argument("--reps", type=int, default=7, help="launches per timed round")
    t.add_argument("--device", type=int, default=0)
    t.add_argument("--cache", help="tile cache file (default: $GOOFY_TILE_CACHE or the per-user cache)")
    args = ap.parse_args(argv)
    return {"run": cmd_run, "encode": cmd_encode, "autotune": cmd_autotune}[args.cmd](args)


if __name__ == "__main__":
    sys.exit(main())
