#!/usr/bin/env python3
"""Builds oracle/_ref/libmsplat_ref.so: the reference's own Metal source for
the per-Gaussian stages, compiled unchanged as host C++ — TEST
INFRASTRUCTURE ONLY (it pins the oracle; nothing in the product uses it).

The reference (semhfe/msplat) is Metal-only, so its kernels cannot run here.
Its per-Gaussian helper functions and the bodies of its per-Gaussian kernels
are plain arithmetic, however: this recipe copies those line ranges of
core/metal/msplat_metal.metal, as they are, into oracle/_ref/ (git-ignored,
never committed) and compiles them against oracle/metal_shim.h (the MSL
types and functions) and oracle/ref_kernels.cpp (a host loop around each
kernel body, with the kernel's own parameter names).

Every range is checked against the text its first and last lines must hold,
so an edited reference fails loudly instead of compiling something else.

Left out on purpose, with the reason:
  * the device-memory overloads of scale_rot_to_cov3d, project_cov3d_ewa,
    cov2d_to_conic_vjp, project_cov3d_ewa_vjp and scale_rot_to_cov3d_vjp
    (lines 180-197, 215-263, 1272-1286, 1302-1372, 1492-1533): with the
    address-space qualifiers gone they would redefine the thread-local
    overloads, which are the ones the fused kernels call;
  * the device-pointer overloads of read_packed_float2/3 (370-372, 393-395),
    for the same reason (the constant-pointer overloads take their calls).

The tile scan and the per-tile sort + pack (prefix_sum_tiles_kernel,
hybrid_sort_pack_kernel) run as single 1024-thread threadgroups on host
threads, their bitonic networks and Hillis-Steele scans as written.

The chunked backward (compute_chunk_prefix_suffix_kernel,
rasterize_backward_chunked_kernel) is compiled but run only where it is
defined: a lane whose pixel has no contributor in a chunk (or lies outside
the image) returns before the kernel's barriers and SIMD-group broadcasts
from lane 0, which is undefined on the GPU when lane 0 is such a lane and
would leave the host emulation's barriers waiting.  ref_kernels.cpp runs it
only when, for every (8x8 threadgroup, chunk), either all of the group's
lanes return there or none does, and reports whether it ran.

The rasterizers and the SSIM kernels use threadgroup memory, barriers and
SIMD-group functions; metal_shim.h runs their threadgroups on host threads.

The host code on the path is copied the same way and compiled by
ref_model.cpp against model_shim.h (host stand-ins for the Model, Camera,
InputData and MTensor types with the members that code uses): from
core/src/model.cpp the seed initialisation (Model::Model, setupOptimizers,
with the k-nearest adapter of core/include/kdtree_tensor.hpp, whose
nanoflann query nanoflann_shim.h answers), the MCMC pass (computeRelocation, relocate,
addNewGaussians, mcmcAfterTrain: lines 311-660), the checkpoint save and
load (696-843), the camera setup (prepareCam, getDownscaleFactor) and the
psnr / l1_loss metrics; from
core/src/ssim.cpp ssim_eval and its blur; the COLMAP binary loader
(loaders/load_colmap.cpp), the point-cloud readers (loaders/load_ply.cpp),
autoScaleAndCenter (input_data.cpp), the Nerfstudio and Polycam loaders
(loaders/load_nerfstudio.cpp, load_polycam.cpp, whose nlohmann::json calls
json_shim.h answers) and the Gaussian PLY / .splat writers and PLY reader
(loaders/save_gaussians.cpp).

Usage: python oracle/ref_build.py [--reference DIR]   (default: /root/reference)
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libmsplat_ref.so")
METAL = os.path.join("core", "metal", "msplat_metal.metal")
MODEL = os.path.join("core", "src", "model.cpp")
SSIM = os.path.join("core", "src", "ssim.cpp")
COLMAP = os.path.join("core", "src", "loaders", "load_colmap.cpp")
PLY = os.path.join("core", "src", "loaders", "load_ply.cpp")
INPUT = os.path.join("core", "src", "input_data.cpp")
SAVE = os.path.join("core", "src", "loaders", "save_gaussians.cpp")
KDTREE = os.path.join("core", "include", "kdtree_tensor.hpp")
IMAGE_IO = os.path.join("core", "src", "loaders", "image_io.cpp")
NERF = os.path.join("core", "src", "loaders", "load_nerfstudio.cpp")
POLY = os.path.join("core", "src", "loaders", "load_polycam.cpp")
# Host code compiled by ref_model.cpp against model_shim.h (host stand-ins
# for Model, Camera and MTensor): (file, first, last, first-line text, last-line text)
HOST_RANGES = [
    (KDTREE, 8, 41, "// nanoflann adapter for a flat float array of 3D points.", "};"),  # PointsTensor (k nearest)
    (MODEL, 21, 31, "static const double C0 = 0.28209479177387814;", "}"),     # C0, numShBases
    (MODEL, 33, 49, "// Metrics on CPU MTensor data", "}"),                      # psnr, l1_loss
    (MODEL, 80, 254, "// Model constructor", "}"),                               # seeds, setupOptimizers
    (MODEL, 276, 282, "int Model::getDownscaleFactor(int step) {", "}"),
    (MODEL, 311, 660, "void Model::computeRelocation(float opacity_old_sig, float* scale_old_exp, int N,", "}"),
    (MODEL, 696, 843, "// ── Checkpoint save/load", "}"),             # saveCheckpoint, loadCheckpoint
    (MODEL, 845, 889, "Model::CamSetup Model::prepareCam(Camera& cam, int step) {", "}"),
    (SSIM, 26, 123, "// Separable Gaussian blur on a single-channel (H, W) image.", "}"),  # gaussianBlur, ssim_eval
    (COLMAP, 7, 165, "namespace fs = std::filesystem;", "}"),               # the COLMAP binary loader
    (PLY, 6, 205, "// Property types in PLY files", "}"),                   # readPly, readColmapPoints
    (INPUT, 81, 111, "void Camera::loadMask(const std::string &maskDir) {", "}"),  # training masks
    (INPUT, 115, 169, "void autoScaleAndCenter(InputData &data) {", "}"),   # pose centring and scaling
    (INPUT, 173, 205, "std::tuple<std::vector<Camera>, Camera*> InputData::getCameras(", "}"),  # --val, --eval split
    (SAVE, 10, 231, "void saveGaussianPly(const std::string &path, GaussianParams &p, int step) {", "}"),  # PLY / .splat
    (NERF, 7, 72, "namespace fs = std::filesystem;", "}"),                  # the Nerfstudio loader
    (POLY, 7, 95, "namespace fs = std::filesystem;", "}"),                  # the Polycam loader
    (IMAGE_IO, 115, 161, "Image resizeArea(const Image &src, int dstW, int dstH) {", "}"),  # area resize
]

# (first line, last line, text of the first line, text of the last line), 1-based, inclusive
HELPER_RANGES = [
    (5, 179, "#define BLOCK_X 16", ""),                    # defines, SH constants, geometry helpers
    (199, 214, "// Thread-local overload: writes cov3d", ""),  # scale_rot_to_cov3d (thread)
    (265, 344, "// Thread-local overload: reads cov3d", "}"),  # project_cov3d_ewa (thread), bounds, project_pix
    (349, 369, "inline int2 read_packed_int2(", ""),       # packed helpers
    (374, 392, "inline void write_packed_float2(", ""),
    (397, 416, "inline float3 read_packed_float3(device const", "}"),
    (620, 776, "void sh_coeffs_to_color(", "}"),           # SH forward and VJP
    (1251, 1271, "// given v_xy_pix, get v_xyz", ""),       # project_pix_vjp
    (1288, 1301, "// Thread-local overload", ""),           # cov2d_to_conic_vjp (thread)
    (1374, 1491, "// Thread-local overload: reads cov3d from registers, writes", ""),  # EWA VJP, quat VJP
    (1535, 1569, "// Thread-local overload: reads v_cov3d", "}"),  # scale_rot_to_cov3d_vjp (thread)
    (1836, 1858, "// Adam update helper", "};"),           # adam_update_element, SHAdamParams
    (2242, 2244, "#define BITONIC_TG_CAP 2048u", "constant constexpr uint64_t SORT_KEY_SENTINEL = 0xFFFFFFFFFFFFFFFFULL;"),
    (2248, 2276, "inline uint next_pow2(uint x) {", "}"),  # pad_count, make_sort_key, gaussian_is_active
    (2278, 2337, "// Hillis-Steele exclusive scan over threadgroup memory.", "}"),  # tile scan, bitonic sorts
    (906, 929, "inline int warp_reduce_all_max(", "}"),   # SIMD-group reductions
    (2771, 2774, "#define SSIM_WIN 11", "#define SSIM_C2 0.0009f"),
    (3376, 3382, "constant float GAUSS_1D[11] = {", "#define SSIM_TG 16   // threadgroup dimension (16×16 = 256 threads)"),
    (3862, 3870, "static inline uint pcg_hash32(", "}"),
]

# kernel name -> parameter names that must appear in its signature (the host
# wrappers in ref_kernels.cpp declare exactly these)
KERNELS = {
    "project_and_sh_forward_kernel": ["num_points", "means3d", "scales", "glob_scale", "quats", "viewmat", "projmat",
                                      "intrins", "img_size", "tile_bounds", "clip_thresh", "xys", "depths", "radii",
                                      "conics", "num_tiles_hit", "degree", "degrees_to_use", "cam_pos",
                                      "features_dc", "features_rest", "colors", "aabb", "nan_counts", "gp"],
    "project_and_sh_backward_kernel": ["num_points", "means3d", "scales", "glob_scale", "quats", "viewmat",
                                       "projmat", "intrins", "img_size", "radii", "conics", "v_xy", "v_depth",
                                       "v_conic", "v_mean3d", "v_scale", "v_quat", "degree", "degrees_to_use",
                                       "cam_pos", "v_colors", "features_dc", "features_rest", "dc_exp_avg",
                                       "dc_exp_avg_sq", "rest_exp_avg", "rest_exp_avg_sq", "adam_hp", "nan_counts",
                                       "idx"],
    "fused_adam_kernel": ["params", "grads", "exp_avg", "exp_avg_sq", "step_size", "beta1", "beta2", "bc2_sqrt",
                          "eps", "n", "nan_counts", "group_idx", "tid"],
    "sgld_noise_gen_kernel": ["noise", "N", "seed", "idx"],
    "sgld_noise_kernel": ["means", "scales", "quats", "opacities", "noise", "N", "noise_lr", "xyz_lr", "max_disp",
                          "idx"],
    "mcmc_reg_grad_kernel": ["opacities", "scales", "v_opacity", "v_scale", "N", "op_reg", "sc_reg", "radii",
                             "invis_scale", "v_dc_sq", "idx"],
    "count_intersections_kernel": ["xys", "radii", "depths", "tile_bounds", "tile_counts", "num_points", "aabb", "gid"],
    "prefix_sum_tiles_kernel": ["tile_counts_in", "exact_offsets", "sort_offsets", "tile_bins", "num_tiles",
                                "capacity", "tile_range", "tid"],
    "hybrid_sort_pack_kernel": ["tile_counts_in", "sort_offsets", "exact_offsets", "isect_keys_unsorted", "xys_in",
                                "conics_in", "opacities_in", "colors_in", "packed_xy_opac", "packed_conic",
                                "packed_rgb", "gaussian_ids", "capacity", "num_points", "nan_counts", "tile_range",
                                "key_capacity", "tg_id", "tid"],
    "scatter_intersections_kernel": ["xys", "depths", "radii", "tile_bounds", "sort_offsets", "tile_write_counters",
                                     "isect_keys_unsorted", "num_points", "aabb", "capacity", "tile_range", "gid"],
    "nd_rasterize_forward_kernel": ["tile_bounds", "img_size", "channels", "tile_bins", "packed_xy_opac",
                                    "packed_conic", "packed_rgb", "final_Ts", "final_index", "out_img", "background",
                                    "blockDim", "tile_range", "blockIdx", "threadIdx", "tr"],
    "rasterize_backward_kernel": ["tile_bounds", "img_size", "gaussian_ids_sorted", "tile_bins", "packed_xy_opac",
                                  "packed_conic", "packed_rgb", "background", "final_Ts", "final_index", "v_output",
                                  "v_xy", "v_conic", "v_rgb", "v_opacity", "tile_range", "gp", "blockIdx", "tr",
                                  "warp_size", "wr"],
    "rasterize_forward_chunked_kernel": ["tile_bounds", "img_size", "channels", "tile_bins", "packed_xy_opac",
                                         "packed_conic", "packed_rgb", "chunk_T", "chunk_C", "chunk_final_idx",
                                         "chunk_size", "K_max", "blockDim", "nan_counts", "blockIdx", "tr"],
    "compute_chunk_prefix_suffix_kernel": ["num_pixels", "K_max", "chunk_T", "chunk_C", "chunk_final_idx",
                                           "prefix_T", "after_C", "img_size", "gp"],
    "rasterize_backward_chunked_kernel": ["tile_bounds", "img_size", "gaussian_ids_sorted", "tile_bins",
                                          "packed_xy_opac", "packed_conic", "packed_rgb", "background", "final_Ts",
                                          "chunk_final_idx", "prefix_T_buf", "chunk_T_buf", "after_C_buf",
                                          "v_output", "v_xy", "v_conic", "v_rgb", "v_opacity", "chunk_size", "K_max",
                                          "gp", "blockIdx", "tr", "warp_size", "wr"],
    "rasterize_forward_merge_kernel": ["num_pixels", "K_max", "chunk_T", "chunk_C", "chunk_final_idx", "final_Ts",
                                       "final_index", "out_img", "background", "img_size", "gp"],
    "ssim_h_fwd_kernel": ["rendered", "gt", "img_size", "ssim_h_buf", "gid", "lid", "tr", "tgid"],
    "ssim_fused_v_fwd_h_bwd_kernel": ["rendered", "gt", "ssim_h_buf", "img_size", "ssim_weight", "inv_n",
                                      "deriv_h_buf", "loss_sum", "nan_counts", "mask", "has_mask", "gid", "lid", "tr",
                                      "tgid", "tg_size"],
    "ssim_v_bwd_kernel": ["rendered", "gt", "ssim_h_buf", "img_size", "ssim_weight", "inv_n", "v_rendered",
                          "nan_counts", "mask", "has_mask", "gid", "lid", "tr", "tgid"],
}


def extract(lines, first, last, head, tail, path=METAL):
    got_head = lines[first - 1].strip()
    got_tail = lines[last - 1].strip()
    if not got_head.startswith(head) or got_tail != tail:
        raise SystemExit(f"{path}:{first}-{last}: expected '{head}' ... '{tail}', found '{got_head}' ... "
                         f"'{got_tail}': the reference changed; review the ranges")
    return f"#line {first} \"{os.path.basename(path)}\"\n" + "".join(lines[first - 1:last])


def kernel_body(lines, name, params):
    start = next((i for i, l in enumerate(lines) if l.startswith(f"kernel void {name}(")), None)
    if start is None:
        raise SystemExit(f"{METAL}: kernel {name} not found")
    open_i = next(i for i in range(start, len(lines)) if lines[i].rstrip() == ") {")
    sig = "".join(lines[start:open_i])
    import re
    for p in params:
        if not re.search(r"\b" + re.escape(p) + r"\b", sig):
            raise SystemExit(f"{METAL}:{start + 1}: parameter {p} of {name} not found")
    close_i = next(i for i in range(open_i + 1, len(lines)) if lines[i].rstrip() == "}")
    return f"#line {open_i + 2} \"msplat_metal.metal\"\n" + "".join(lines[open_i + 1:close_i]), (start + 1, close_i + 1)


def build(reference: str, quiet: bool = False) -> str:
    src = os.path.join(reference, METAL)
    if not os.path.exists(src):
        raise SystemExit(f"{src} not found")
    with open(src) as f:
        lines = f.readlines()
    os.makedirs(OUT, exist_ok=True)
    helpers = "// extracted by oracle/ref_build.py from " + METAL + " (not committed)\n"
    helpers += "".join(extract(lines, *r) for r in HELPER_RANGES)
    with open(os.path.join(OUT, "ref_helpers.inc"), "w") as f:
        f.write(helpers)
    spans = {}
    for name, params in KERNELS.items():
        body, span = kernel_body(lines, name, params)
        spans[name] = span
        with open(os.path.join(OUT, f"k_{name}.inc"), "w") as f:
            f.write(body)
    host = "// extracted by oracle/ref_build.py from the reference's host sources (not committed)\n"
    sources = {}
    for path, first, last, head, tail in HOST_RANGES:
        if path not in sources:
            full = os.path.join(reference, path)
            if not os.path.exists(full):
                raise SystemExit(f"{full} not found")
            with open(full) as f:
                sources[path] = f.readlines()
        host += extract(sources[path], first, last, head, tail, path=path)
    with open(os.path.join(OUT, "model_host.inc"), "w") as f:
        f.write(host)
    cxx = shutil.which("g++") or "c++"
    cmd = [cxx, "-O2", "-std=c++20", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-Wno-unknown-pragmas", "-pthread", "-I", HERE, "-I", OUT, os.path.join(HERE, "ref_kernels.cpp"),
           os.path.join(HERE, "ref_model.cpp"), "-o", LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise SystemExit(f"compile failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if not quiet:
        for name, (a, b) in spans.items():
            print(f"{name}: {METAL}:{a}-{b}")
        for path, first, last, _, _ in HOST_RANGES:
            print(f"host code: {path}:{first}-{last}")
        print(LIB)
    return LIB


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    a = ap.parse_args()
    build(a.reference)
    return 0


if __name__ == "__main__":
    sys.exit(main())
