#!/usr/bin/env python
"""Benchmark: frames/s (and Gpix/s) of the 1080p 4x MSAA textured workload.

Workload ("c2"): 1920x1080 RGBA8, 4x MSAA, RG32F depth-stencil (the
reference's depth format), a 317x317-vertex height-field grid (199,712
triangles) in 8 indexed draws; one 2048^2 RGBA8 value-noise texture with a
12-level box mip chain, trilinear on even draws and 16x anisotropic on odd
draws; src-alpha blending; depth LESS; clear + 8 draws + MSAA resolve per
frame.  Inputs are synthetic and seeded (numpy PCG64, seed 20261204).

One step = one frame.  `value` times the frame with every input resident in
HBM (CUDA events on the renderer's stream, L2 flushed between steps with a
256 MiB write); `e2e` times the same frame through the C ABI from pinned
host memory: vertex and index upload, the frame, and the download of the
resolved image.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

--impl reference times the reference's CPU path on the host cores: the
CPU restatement of the reference renderer (oracle/), one frame per process
across all host cores.  Multi-GPU runs are replicas (each rank renders its own
frames; no data exchange).
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "frames/s at 1920x1080 4xMSAA (textured trilinear+16xAF, src-alpha blend, 199,712 tris)"
UNIT = "frames/s"
SEED = 20261204


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--no-uneven", action="store_true", help="skip the 256-frame batched-draw leg")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-filter leg")
    ap.add_argument("--no-facade", action="store_true", help="skip the C++ facade leg")
    ap.add_argument("--no-autotune", action="store_true", help="time under the default scheduling parameters")
    ap.add_argument("--no-ingest", action="store_true", help="skip the texture / mesh ingest leg")
    ap.add_argument("--no-sasl", action="store_true", help="skip the SASL-compiled pixel shader leg")
    ap.add_argument("--cpu-configs", action="store_true",
                    help="time the CPU restatement (and the reference, where built) on the five workloads")
    ap.add_argument("--size", default="1920x1080",
                    help="render-target size; smaller sizes are for profiling captures only")
    return ap.parse_args()


def workload_config(scene):
    return {"workload": "c2_1080p_4xmsaa_textured_af16_blend", "width": scene.width,
            "height": scene.height, "samples": scene.samples, "triangles": scene.triangles,
            "draws": len(scene.draws), "texture": "2048x2048 RGBA8 + 11 mips",
            "depth_format": "RG32F", "l2": "flushed between steps (256 MiB write)",
            "seed": SEED}


# ---------------------------------------------------------------------------
# algorithmic bytes (every item counted once)
DS_BYTES = 8       # RG32F depth-stencil element
DEPTH_WORD = 4     # the depth word of it that early-Z reads and writes
COLOR_BYTES = 4    # RGBA8
STAGED_REC = 7 * 16  # edge equations, bbox, base and two gradients of the position
FRAG_REC = 12        # record index, position, coverage per quad


def frame_bytes(scene):
    """Per frame: geometry + sampled texture + framebuffer traffic (clears,
    depth and colour read-modify-write, resolve)."""
    npx = scene.width * scene.height
    s = scene.samples
    geom = sum(v.nbytes for v in scene.buffers.values())
    tex = 0
    for img, mips in scene.textures.values():
        tex += img.nbytes * 4 // 3 if mips else img.nbytes
    fb = (npx * s * (COLOR_BYTES + DS_BYTES)          # clears
          + 2 * npx * s * DEPTH_WORD                  # depth read-modify-write
          + 2 * npx * s * COLOR_BYTES                 # colour read-modify-write (blend)
          + npx * s * COLOR_BYTES + npx * COLOR_BYTES)  # resolve
    return geom + tex + fb


def cover_bytes(scene, stats):
    """Per frame, k_cover: the depth words read and written once, one staged
    triangle record per clipped primitive, one fragment record per quad."""
    npx = scene.width * scene.height
    cprims = sum(st["cprimitives"] for st in stats)
    quads = sum(st["ps_invocations"] for st in stats) // 4
    return 2 * npx * scene.samples * DEPTH_WORD + cprims * STAGED_REC + quads * FRAG_REC


def read_traffic():
    """Per-launch DRAM traffic of k_cover2 from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "pass_kernels_c2_1080p_4x.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def measured_peak():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    def __init__(self, index):
        self.index, self.samples, self.proc = index, [], None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for s in self.samples for n, v in zip(names, s[4:8]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons}


# ---------------------------------------------------------------------------
def cpu_oracle_fps(scene_kw, frames=1):
    """The CPU restatement on one host core: seconds for `frames` full frames."""
    from salviarenderer_gb300 import abi, Device, scenes
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    lib = abi.bind(ctypes.CDLL(os.path.join(ROOT, "oracle", "_build", "libsg_oracle.so")))
    dev = Device(lib)
    scene = scenes.c2_scene(**scene_kw)
    b = scenes.Bound(dev, scene)
    b.frame()
    t0 = time.perf_counter()
    for _ in range(frames):
        b.frame()
    return time.perf_counter() - t0


_WORKER = {}


def _worker_init(scene_kw):
    from salviarenderer_gb300 import abi, Device, scenes
    lib = abi.bind(ctypes.CDLL(os.path.join(ROOT, "oracle", "_build", "libsg_oracle.so")))
    dev = Device(lib)
    _WORKER["b"] = scenes.Bound(dev, scenes.c2_scene(**scene_kw))
    _WORKER["dev"] = dev


def _worker_frame(_):
    t0 = time.perf_counter()
    _WORKER["b"].frame()
    return time.perf_counter() - t0


def run_reference(args):
    """CPU reference arm: the restatement, one frame per process on every core."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    from salviarenderer_gb300 import scenes
    cores = os.cpu_count() or 1
    kw = dict(seed=SEED)
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_worker_init, initargs=(kw,)) as pool:
        for _ in range(args.warmup):
            pool.map(_worker_frame, range(cores))
        t0 = time.perf_counter()
        for _ in range(args.steps):
            pool.map(_worker_frame, range(cores))
        dt = time.perf_counter() - t0
    fps = args.steps * cores / dt
    scene = scenes.c2_scene(**kw)
    line = {"impl": "reference", "metric": METRIC, "value": fps, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "config": workload_config(scene),
            "cpu_baseline": {"value": fps, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{cores} full frames per step, one per process"},
            "e2e": {"value": fps, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_cpu_configs(args):
    """CPU time of the five workloads, for the CPU-baseline table: the
    restatement (oracle/, one core) everywhere, and the reference renderer
    itself (oracle/_ref, all its worker threads) where it was built (an
    x86-64 host with the reference's sources; C1 and C2 only, as the others
    use extension formats).  Bounded samples: C1 and C2 whole frames; C3 the first 16 of its 256 frames; C5 a clear + resolve
    frame and a frame of 10 of its 1000 instances, extrapolated linearly to
    1000 instances."""
    from salviarenderer_gb300 import abi, Device, scenes
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    libs = {"port": os.path.join(ROOT, "oracle", "_build", "libsg_oracle.so")}
    ref = os.path.join(ROOT, "oracle", "_ref", "libsalvia_ref.so")
    if os.path.exists(ref):
        libs["reference"] = ref

    def seconds(fn, reps=1):
        fn()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        return (time.perf_counter() - t0) / reps

    out = {"host": {"cores": os.cpu_count(), "machine": os.uname().machine}}
    try:
        with open("/proc/cpuinfo") as f:
            names = [l.split(":", 1)[1].strip() for l in f if l.lower().startswith(("model name", "cpu part"))]
        out["host"]["cpu"] = names[0] if names else None
    except OSError:
        pass
    for kind, path in libs.items():
        dev = Device(abi.bind(ctypes.CDLL(path)))
        r = {"cores": 1 if kind == "port" else os.cpu_count()}
        b = scenes.Bound(dev, scenes.c1_scene(seed=SEED))
        r["c1_frames_per_s"] = 1.0 / seconds(b.frame, 3)
        b = scenes.Bound(dev, scenes.c2_scene(seed=SEED))
        r["c2_frames_per_s"] = 1.0 / seconds(b.frame)
        if kind == "reference":  # C3 and C5 use the extension formats (D24S8, RGBA16F, D32F)
            out[kind] = r
            continue
        batch = scenes.UnevenBatch(seed=SEED)
        k = 16
        batch.frames = batch.frames[:k]
        batch.vb = batch.vb[:3 * sum(f["ntris"] for f in batch.frames)]
        u = scenes.BoundUneven(dev, batch)
        t = seconds(u.render_plain)
        r["c3_sample"] = {"frames": k, "triangles": batch.triangles, "pixels": batch.pixels,
                          "frames_per_s": k / t, "mtris_per_s": batch.triangles / t / 1e6}
        t0 = seconds(scenes.Bound(dev, scenes.c5_scene(seed=SEED, instances=0)).frame)
        ki = 10
        tk = seconds(scenes.Bound(dev, scenes.c5_scene(seed=SEED, instances=ki)).frame)
        r["c5_frames_per_s_extrapolated"] = 1.0 / (t0 + (tk - t0) * 1000 / ki)
        r["c5_sample"] = {"instances": ki, "clear_resolve_s": t0, "frame_s": tk}
        out[kind] = r
    print(json.dumps({"cpu_configs": out}), flush=True)


# ---------------------------------------------------------------------------
def time_steps(stream, flush, steps, fn):
    """CUDA-event time of `steps` calls of fn on `stream`, L2 flushed before each."""
    import torch
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for i in range(steps):
        flush.zero_()
        starts[i].record(stream)
        fn()
        ends[i].record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / 1000.0


def measure_uneven(dev, stream, flush, args):
    """The batched-draw workload: 256 frames of uneven size and triangle
    count in one command list, plain (clear + one sg_draw per draw, frame by
    frame) against batched (the list recorded as one CUDA graph)."""
    from salviarenderer_gb300 import scenes
    batch = scenes.UnevenBatch(seed=SEED)
    b = scenes.BoundUneven(dev, batch)
    cl = b.commands()
    dev.submit(cl, stats=True)  # sizes the scratch
    steps = max(1, min(args.steps, 3))
    for _ in range(args.warmup):
        b.render_plain()
    dev.sync()
    plain_s = time_steps(stream, flush, steps, b.render_plain)
    graph = dev.graph_create(cl)
    info = graph.info()
    for _ in range(args.warmup):
        graph.launch()
    dev.sync()
    graph_s = time_steps(stream, flush, steps, graph.launch)
    dev.sync()
    graph.close()
    nf = len(batch.frames)
    return {"workload": "256 frames, sides {256,512,1024,2048}, 1k-500k triangles log-uniform, RGBA8 + D24S8, "
                        "1/3 flat, 2/3 textured (1024^2 trilinear), 1/4 with a stencil-mirror pass",
            "frames": nf, "triangles": batch.triangles, "pixels": batch.pixels,
            "plain_frames_per_s": nf * steps / plain_s, "batched_frames_per_s": nf * steps / graph_s,
            "batched_gpix_per_s": batch.pixels * steps / graph_s / 1e9,
            "batched_over_plain": plain_s / graph_s, "graph_passes": info["passes"],
            "graph_kernels": info["kernels"], "steps": steps}


AF_MLP_FLOPS = 2 * (32 * 64 + 64 * 64 + 64 * 16)  # per lookup, as the tensor cores run the padded layers
AF_TRAIN_FLOPS = AF_MLP_FLOPS + 2 * (16 * 64 + 64 * 64) + 2 * 128 * (80 + 64 + 80)  # fwd + bwd + weight grads


def measure_learned(dev, stream, flush, args, width, height):
    """The learned anisotropic filter: trained on the device from the plain
    16x sampler over 4096 procedural 512^2 textures (20M samples), then the
    1080p frame rendered with its anisotropic draws on the learned filter
    against the plain sampler: frames/s (recorded graphs), PSNR and largest
    error of the resolved image, and the anisotropic pixels' shading
    throughput on the same frame with every draw anisotropic."""
    import numpy as np
    from salviarenderer_gb300 import abi, scenes
    from salviarenderer_gb300.device import AfModel
    t0 = time.perf_counter()
    train = scenes.AfTextures(dev, count=4096, size=512, seed=SEED)
    dev.sync()
    make_s = time.perf_counter() - t0
    model = AfModel(dev, seed=SEED)
    rep = model.train(train.samplers, samples=20_000_000, batch=8192, epochs=2, lr=2e-3, seed=SEED)
    learned = (0.5, 16.0, 0.0)  # confidence threshold, probe range (0, 16]
    steps = max(1, min(args.steps, 10))

    def frame(stride, lrn):
        b = scenes.Bound(dev, scenes.c2_scene(seed=SEED, width=width, height=height, learned=lrn,
                                              af_stride=stride), model if lrn else None)
        cl = b.commands()
        st = [x for x, c in zip(dev.submit(cl, stats=True), cl._cmds) if c.type == abi.CMD_DRAW]
        img = b.outputs()["resolved"]
        g = dev.graph_create(cl)
        for _ in range(args.warmup):
            g.launch()
        dev.sync()
        sec = time_steps(stream, flush, steps, g.launch)
        g.close()
        dev.profile_enable(True)
        dev.profile_read()
        for _ in range(steps):
            dev.submit(cl)
        dev.sync()
        prof = dev.profile_read()
        dev.profile_enable(False)
        af_pixels = sum(x["ps_invocations"] for i, x in enumerate(st) if i % stride == stride - 1)
        return {"fps": steps / sec, "img": img, "shade_ms": prof["shade_ms"] / steps,
                "lookups": prof["af_lookups"] / steps, "fallbacks": prof["af_fallbacks"] / steps,
                "af_pixels": af_pixels}

    def psnr(a, b):
        d = a.astype(np.float64) / 255.0 - b.astype(np.float64) / 255.0
        mse = float((d * d).mean())
        return float("inf") if mse == 0 else 10.0 * math.log10(1.0 / mse)

    out = {"training": {"textures": 4096, "texture_size": 512, "make_textures_s": make_s,
                        "samples": 20_000_000, "batch": 8192, "epochs": 2, "steps": rep["steps"],
                        "first_loss": rep["first_loss"], "last_loss": rep["last_loss"],
                        "train_ms": rep["train_ms"],
                        "samples_per_s": 40_000_000 / (rep["train_ms"] / 1000.0),
                        "tensor_tflops": 40_000_000 * AF_TRAIN_FLOPS / (rep["train_ms"] / 1000.0) / 1e12},
           "filter": {"confidence_threshold": learned[0], "probe_range": [learned[2], learned[1]]}}
    for stride, key in ((2, "c2_frame"), (1, "all_af_frame")):
        p, l = frame(stride, None), frame(stride, learned)
        err = int(np.abs(l["img"].astype(np.int16) - p["img"].astype(np.int16)).max())
        out[key] = {
            "af_draws": "every other draw" if stride == 2 else "all 8 draws",
            "plain_frames_per_s": p["fps"], "learned_frames_per_s": l["fps"],
            "learned_over_plain": l["fps"] / p["fps"],
            "psnr_db": psnr(l["img"], p["img"]), "max_abs_error_lsb": err,
            "af_pixels": p["af_pixels"], "network_lookups": l["lookups"],
            "fallback_rate": l["fallbacks"] / max(1.0, l["lookups"]),
            "shade_ms": {"plain": p["shade_ms"], "learned": l["shade_ms"]},
            "af_gpix_per_s_shade_stage": {"plain": p["af_pixels"] / p["shade_ms"] / 1e6,
                                          "learned": p["af_pixels"] / l["shade_ms"] / 1e6}}
    try:
        out["c5_frame"] = measure_c5(dev, stream, flush, args, model)
    finally:
        model.close()
    return out


def measure_c5(dev, stream, flush, args, model):
    """The large instanced frame: 3840x2160 RGBA16F, 4x MSAA, D32F, 1000
    icosphere instances (5.12M triangles) with morph + vertex-texture
    displacement, 8x anisotropic texturing on the plain sampler and on the
    learned filter; frames/s of each as a recorded graph."""
    import numpy as np
    from salviarenderer_gb300 import scenes
    steps = max(1, min(args.steps, 5))
    out = {"workload": "3840x2160 RGBA16F 4xMSAA D32F, 1000 instances x 5120 triangles, morph + R32F "
                       "vertex-texture displacement, 2048^2 RGBA8 8x AF, 10% additive"}
    imgs = {}
    for key, lrn in (("plain", None), ("learned", (0.5, 16.0, 0.0))):
        b = scenes.Bound(dev, scenes.c5_scene(seed=SEED, learned=lrn), model if lrn else None)
        cl = b.commands()
        dev.submit(cl)
        dev.sync()
        imgs[key] = np.frombuffer(b.outputs()["resolved"], dtype=np.float16).astype(np.float32)
        g = dev.graph_create(cl)
        for _ in range(args.warmup):
            g.launch()
        dev.sync()
        sec = time_steps(stream, flush, steps, g.launch)
        g.close()
        out[key + "_frames_per_s"] = steps / sec
        out["triangles"] = b.scene.triangles
    d = imgs["learned"] - imgs["plain"]
    peak = float(np.abs(imgs["plain"]).max())
    out["psnr_db_vs_plain"] = 10.0 * math.log10(peak * peak / max(float((d * d).mean()), 1e-30))
    out["max_abs_error"] = float(np.abs(d).max())
    out["learned_over_plain"] = out["learned_frames_per_s"] / out["plain_frames_per_s"]
    return out


def measure_facade(args, scene, resolved_want):
    """The same frame through the C++ facade (include/salvia_gb300/renderer.hpp)
    as a reference application drives it: tests/cpp/facade_scene.cpp, built
    against the library, issues clears, one draw_index per draw, resolve and
    flush each frame; the facade queues the calls and submits them as one
    command list at flush.  Wall time per frame up to the end of its flush
    (L2 flushed before each frame), and whether its resolved image equals
    the recorded graph's."""
    import tempfile
    from salviarenderer_gb300 import scenes
    from salviarenderer_gb300 import build as pbuild
    libdir, libfile = os.path.split(pbuild.ensure_built())
    with tempfile.TemporaryDirectory() as tmp:
        exe, inp, out = (os.path.join(tmp, n) for n in ("facade_scene", "in.bin", "out.bin"))
        subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "facade_scene.cpp"), "-o", exe, "-L", libdir,
                        f"-l{libfile[3:-3]}", f"-Wl,-rpath,{libdir}"], check=True)
        scenes.write_facade_input(scene, inp)
        run = subprocess.run([exe, inp, out, str(args.steps), str(args.warmup)], check=True,
                             capture_output=True, text=True)
        ms = float(next(l for l in run.stdout.splitlines() if l.startswith("facade_ms_per_frame")).split()[1])
        raw = open(out, "rb").read()
    n = scene.width * scene.height
    off = n * scene.samples * (4 + 8)
    return {"frames_per_s": 1000.0 / ms, "ms_per_frame": ms,
            "calls_per_frame": "clear_color, clear_depth_stencil, 8 x (set_pixel_shader, draw_index), resolve, flush",
            "resolved_equals_graph": raw[off:off + n * 4] == bytes(resolved_want)}


# The anisotropic draws' pixel shader in SASL: tex2D (sample_2d_grad with the
# coordinate's quad differences) modulated by the colour, SG_PS_TEX_GRAD_MODULATE's
# arithmetic.
SASL_GRAD_PS = """
sampler s;
struct PSIn {
    float4 uv:    TEXCOORD0;
    float4 color: COLOR0;
};
float4 ps_main(PSIn in): COLOR {
    return tex2D(s, in.uv.xy) * in.color;
}
"""


def measure_sasl(dev, stream, flush, args, width, height):
    """The 1080p frame with its anisotropic draws' pixel shader compiled from
    SASL (sg_sasl_translate -> a user shader module built with nvcc) against
    the stock program: translate + build time, frames/s of both (recorded
    graphs) and whether the resolved images are equal."""
    import tempfile
    import numpy as np
    from salviarenderer_gb300 import abi, sasl, scenes
    t0 = time.perf_counter()
    obj = sasl.compile(dev.lib, SASL_GRAD_PS, sasl.LANG_PIXEL_SHADER, cls="bench_sasl_grad_ps")
    sasl.load(sasl.build_module([obj], tempfile.mkdtemp(prefix="sasl_bench_")))
    build_s = time.perf_counter() - t0
    steps = max(1, min(args.steps, 10))

    def frame(use_sasl):
        sc = scenes.c2_scene(seed=SEED, width=width, height=height)
        if use_sasl:
            for d in sc.draws:
                if d["ps"]["program"] == abi.PS_TEX_GRAD_MODULATE:
                    d["ps"] = dict(d["ps"], program=obj.program)
        b = scenes.Bound(dev, sc)
        cl = b.commands()
        dev.submit(cl)
        img = b.outputs()["resolved"]
        g = dev.graph_create(cl)
        for _ in range(args.warmup):
            g.launch()
        dev.sync()
        sec = time_steps(stream, flush, steps, g.launch)
        g.close()
        return steps / sec, img

    fs, a = frame(False)
    fu, b = frame(True)
    return {"shader": "tex2D(s, in.uv.xy) * in.color on the 4 anisotropic draws", "translate_and_build_s": build_s,
            "stock_frames_per_s": fs, "sasl_frames_per_s": fu, "sasl_over_stock": fu / fs,
            "resolved_equal": bool(np.array_equal(a, b))}


def synthetic_obj(path, n):
    """An n x n height-field grid as a Wavefront OBJ file: positions,
    texcoords and normals per grid point, two triangles per cell with
    v/vt/vn corners, the two halves in two materials."""
    import numpy as np
    rng = np.random.default_rng(SEED)
    ax = np.linspace(-1.0, 1.0, n + 1, dtype=np.float32)
    x, y = np.meshgrid(ax, ax)
    z = rng.uniform(-0.05, 0.05, size=x.shape).astype(np.float32)
    with open(path, "w") as f:
        f.write("mtllib grid.mtl\n")
        f.write("".join(f"v {a:.6f} {b:.6f} {c:.6f}\n" for a, b, c in zip(x.ravel(), y.ravel(), z.ravel())))
        f.write("".join(f"vt {a * 0.5 + 0.5:.5f} {b * 0.5 + 0.5:.5f}\n" for a, b in zip(x.ravel(), y.ravel())))
        f.write("vn 0 0 1\n")
        for half, name in ((0, "left"), (1, "right")):
            f.write(f"usemtl {name}\n")
            rows = []
            for r in range(n):
                for c in range(half * n // 2, (half + 1) * n // 2):
                    a, b, d, e = (r * (n + 1) + c + 1, r * (n + 1) + c + 2, (r + 1) * (n + 1) + c + 1,
                                  (r + 1) * (n + 1) + c + 2)
                    rows.append(f"f {a}/{a}/1 {b}/{b}/1 {e}/{e}/1\nf {a}/{a}/1 {e}/{e}/1 {d}/{d}/1\n")
            f.write("".join(rows))
    with open(os.path.join(os.path.dirname(path), "grid.mtl"), "w") as f:
        f.write("newmtl left\nKd 0.8 0.2 0.2\nnewmtl right\nKd 0.2 0.8 0.2\n")
    return 2 * n * n


def measure_ingest(dev, stream, args):
    """Texture and mesh ingest (tex_io.cpp, mesh_io_obj.cpp): the library's
    host PNG codec on a 2048^2 RGBA value-noise image, load_texture end to
    end (decode, upload, device conversion) into RGBA8 and RGBA32F, and the
    OBJ loader on a 512 x 512-cell grid (524,288 faces)."""
    import tempfile
    import numpy as np
    from salviarenderer_gb300 import abi, ingest, scenes
    reps = max(2, min(args.steps, 5))
    img = scenes.to_rgba8(scenes.value_noise(np.random.default_rng(SEED), 2048))[::-1].copy()
    t0 = time.perf_counter()
    for _ in range(reps):
        png = ingest.encode_png(dev.lib, img)
    enc_s = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        got = ingest.decode_image(dev.lib, png)
    dec_s = (time.perf_counter() - t0) / reps
    assert np.array_equal(got, img)
    out = {"image": "2048x2048 RGBA8 value noise", "png_bytes": len(png),
           "png_encode_mpix_per_s": img.shape[0] * img.shape[1] / enc_s / 1e6,
           "png_decode_mpix_per_s": img.shape[0] * img.shape[1] / dec_s / 1e6,
           "png_decode_mb_per_s": len(png) / dec_s / 1e6}
    for fmt, name in ((abi.FMT_RGBA8, "rgba8"), (abi.FMT_RGBA32F, "rgba32f")):
        tex = dev.texture(2048, 2048, 1, fmt)
        ingest.write_image(dev, tex, img)
        dev.sync()
        t0 = time.perf_counter()
        for _ in range(reps):
            ingest.write_image(dev, tex, img)
        dev.sync()
        w_s = (time.perf_counter() - t0) / reps
        t0 = time.perf_counter()
        for _ in range(reps):
            dev.texture_destroy(ingest.load_texture(dev, png, fmt))
        dev.sync()
        l_s = (time.perf_counter() - t0) / reps
        out[f"write_image_{name}_ms"] = w_s * 1e3
        out[f"load_texture_{name}_ms"] = l_s * 1e3
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "grid.obj")
        faces = synthetic_obj(path, 512)
        size = os.path.getsize(path)
        t0 = time.perf_counter()
        for _ in range(reps):
            data = ingest.load_obj(dev.lib, path, False)
        obj_s = (time.perf_counter() - t0) / reps
        t0 = time.perf_counter()
        meshes = ingest.create_mesh_from_obj(dev, path, False)
        dev.sync()
        mesh_s = time.perf_counter() - t0
    out.update({"obj": "512x512-cell grid, v/vt/vn corners, 2 materials", "obj_bytes": size, "obj_faces": faces,
                "obj_vertices": int(data.vertices.shape[0]), "obj_meshes": len(meshes),
                "obj_load_mb_per_s": size / obj_s / 1e6, "obj_load_mfaces_per_s": faces / obj_s / 1e6,
                "create_mesh_from_obj_ms": mesh_s * 1e3})
    return out


def run_gpu(args):
    import torch
    import torch.distributed as dist
    from salviarenderer_gb300 import abi, Device, scenes
    from salviarenderer_gb300 import build as pbuild

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    # a dedicated stream: the renderer and the timing events share it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    lib = abi.bind(ctypes.CDLL(pbuild.ensure_built()))
    dev = Device(lib, cuda_device=local, stream=stream.cuda_stream)
    width, height = (int(v) for v in args.size.lower().split("x"))
    scene = scenes.c2_scene(seed=SEED + rank, width=width, height=height)
    b = scenes.Bound(dev, scene)
    cl = b.commands()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    def max_over_ranks(x):
        if world > 1:
            t = torch.tensor([x], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            x = float(t.item())
        return x

    # pipeline counters of one frame (untimed), then the autotuner's pick of
    # the scheduling parameters for this frame (sg_autotune; untimed)
    frame_stats = [st for st, c in zip(dev.submit(cl, stats=True), cl._cmds) if c.type == abi.CMD_DRAW]
    tuning = dev.get_tuning() if args.no_autotune else dev.autotune(cl, reps=3)[0]

    # plain path: one sg_draw (one kernel chain) per draw, as the reference's API is called
    for _ in range(args.warmup):
        b.frame()
    barrier()
    plain_s = max_over_ranks(time_steps(stream, flush, args.steps, b.frame))

    # batched: the frame as one command list, recorded once into a CUDA graph
    graph = dev.graph_create(cl)
    ginfo = graph.info()
    for _ in range(args.warmup):
        graph.launch()
    barrier()
    with ClockSampler(local) as clk:
        graph_s = max_over_ranks(time_steps(stream, flush, args.steps, graph.launch))
    dev.sync()
    # the same list submitted each frame (sg_submit), with per-stage timing
    for _ in range(args.warmup):
        dev.submit(cl)
    dev.sync()
    dev.profile_enable(True)
    barrier()
    submit_s = max_over_ranks(time_steps(stream, flush, args.steps, lambda: dev.submit(cl)))
    prof = dev.profile_read()
    dev.profile_enable(False)
    frames = args.steps * world
    fps = frames / graph_s

    # end to end through the C ABI from pinned host memory: vertex and index
    # upload, the recorded frame, the resolved image back
    vb_host = torch.from_numpy(scene.buffers["vb"]).pin_memory()
    ib_host = torch.from_numpy(scene.buffers["ib"]).pin_memory()
    out_bytes = scene.width * scene.height * 4
    res_host = torch.empty(out_bytes, dtype=torch.uint8).pin_memory()
    vb_h, ib_h = b.buf["vb"], b.buf["ib"]

    def e2e_frame():
        lib.sg_buffer_upload(dev.handle, vb_h, 0, ctypes.c_void_p(vb_host.data_ptr()), vb_host.numel() * 4)
        lib.sg_buffer_upload(dev.handle, ib_h, 0, ctypes.c_void_p(ib_host.data_ptr()), ib_host.numel() * 4)
        graph.launch()
        st = lib.sg_texture_download(dev.handle, b.resolved, 0, ctypes.c_void_p(res_host.data_ptr()), out_bytes)
        if st != abi.SG_OK:
            raise RuntimeError("sg_texture_download failed")

    e2e_fps = None
    if not args.no_e2e:
        for _ in range(args.warmup):
            e2e_frame()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            e2e_frame()
        barrier()
        e2e_fps = frames / max_over_ranks(time.perf_counter() - t0)
    dev.sync()
    facade = None
    if rank == 0 and not args.no_facade and scene.samples > 1:
        graph.launch()
        facade = measure_facade(args, scene, b.outputs()["resolved"])
    uneven = None if args.no_uneven else measure_uneven(dev, stream, flush, args)
    learned = None if args.no_learned else measure_learned(dev, stream, flush, args, width, height)
    ingest_leg = None if (args.no_ingest or rank != 0) else measure_ingest(dev, stream, args)
    sasl_leg = None if (args.no_sasl or rank != 0) else measure_sasl(dev, stream, flush, args, width, height)

    if rank == 0:
        peak, peak_kind = measured_peak()
        cover_launch_ms = prof["cover_ms"] / max(1, prof["raster_launches"])
        cover_launch_bytes = cover_bytes(scene, frame_stats)  # one pass per frame: one coverage launch
        achieved = cover_launch_bytes / (cover_launch_ms / 1000.0) / 1e9
        fbytes = frame_bytes(scene)
        frame_achieved = fbytes / (graph_s / args.steps) / 1e9
        cpu = None
        if not args.no_cpu_baseline:
            frames_cpu = 2
            dt = cpu_oracle_fps(dict(seed=SEED), frames=frames_cpu)
            cpu = {"value": frames_cpu / dt, "unit": UNIT, "cores": 1, "kind": "port",
                   "sample": f"{frames_cpu} full frames of the same workload, single-threaded CPU restatement"}
        line = {
            "metric": METRIC, "value": fps, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * graph_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded height-field grid + value-noise texture)",
            "config": dict(workload_config(scene), parallelism=f"replicas x{world}",
                           path="frame recorded as one CUDA graph (sg_graph_launch)"),
            "paths_frames_per_s": {"plain_per_draw": frames / plain_s, "submitted_list": frames / submit_s,
                                   "recorded_graph": fps,
                                   "cpp_facade": None if facade is None else facade["frames_per_s"]},
            "facade": facade,
            "sasl": sasl_leg,
            "gpix_per_s": fps * scene.width * scene.height / 1e9,
            "gsamples_per_s": fps * scene.width * scene.height * scene.samples / 1e9,
            "mtris_per_s": fps * scene.triangles / 1e6,
            "stage_ms_per_frame": {k: prof[k + "_ms"] / args.steps
                                   for k in ("geometry", "binning", "cover", "shade", "merge")},
            "cover_work_per_frame": {"items": 4 * ((scene.width + 63) // 64) * ((scene.height + 63) // 64),
                                     "batches": prof["cover_batches"] / args.steps,
                                     "rounds": prof["cover_rounds"] / args.steps,
                                     "pairs": prof["cover_pairs"] / args.steps},
            "roofline": {"bound": "hbm", "kernel": "k_cover2", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": read_traffic() if (width, height) == (1920, 1080) else None,
                         "algorithmic_bytes_per_launch": cover_launch_bytes,
                         "launch_ms": cover_launch_ms},
            "frame_roofline": {"algorithmic_bytes_per_frame": fbytes, "achieved": frame_achieved,
                               "peak": peak, "unit": "GB/s", "frac": frame_achieved / peak},
            "pipeline_counters_per_frame": {k: sum(st[k] for st in frame_stats)
                                            for k in frame_stats[0]},
            "cpu_baseline": cpu,
            "e2e": None if e2e_fps is None else {
                "value": e2e_fps, "unit": UNIT,
                "h2d_bytes_per_step": int(vb_host.numel() * 4 + ib_host.numel() * 4),
                "d2h_bytes_per_step": out_bytes},
            "tuning": tuning,
            "autotune": None if args.no_autotune else {
                "searched": dev.autotune_space(), "chosen": {k: tuning[k] for k in dev.autotune_space()},
                "not_searched": {"binning tile": "64x64: the reference's 64/16/4 classification decides edge samples",
                                 "shade_quads_per_warp": "8 by construction (4 lanes per quad)",
                                 "bin_capacity, frag_chunks": "sized from counters, grown after an overflow"}},
            "uneven_batch": uneven,
            "learned_filter": learned,
            "ingest": ingest_leg,
            "gpu_launches": int(ginfo["kernels"]) * args.steps,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    graph.close()
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def main():
    args = parse()
    if args.cpu_configs:
        run_cpu_configs(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
