// Dataset ingestion on the host: the three on-disk layouts the reference
// reads (COLMAP, Nerfstudio, Polycam; core/src/input_data.cpp:244-261 and
// core/src/loaders/), their point clouds, and the image decoding they need
// (PNG, baseline JPEG, binary PPM/PGM), with the reference's area downscale
// and 8-bit quantisation.  No third-party code: a JSON reader, DEFLATE,
// PNG un-filtering and a baseline JPEG decoder are written here.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace msplat {
namespace io {

struct Image {
    int width = 0, height = 0;
    std::vector<float> rgb;   // [H,W,3] in [0, 1]
    bool empty() const { return width <= 0 || height <= 0; }
};

// PNG (8/16-bit grey, grey+alpha, RGB, RGBA, palette; not interlaced),
// baseline/extended-sequential Huffman JPEG, binary PPM (P6) and PGM (P5).
// Throws std::runtime_error with the reason on anything else.
Image read_image(const std::string &path);

// Box-filter resize by fractional pixel coverage (image_io.cpp:115-161).
Image resize_area(const Image &src, int dst_w, int dst_h);

// Remaps a distorted image (OpenCV radial-tangential k1, k2, k3, p1, p2) to
// the undistorted pinhole image with the same intrinsics and size; samples
// that fall outside the source are black.
Image undistort(const Image &src, float fx, float fy, float cx, float cy, float k1, float k2, float p1, float p2,
                float k3);

struct LoadedCamera {
    std::string path;            // image file
    std::string relative_name;   // COLMAP: name under the image folder (mask lookup); else empty
    int width = 0, height = 0;   // from the metadata; 0 = take the image's
    float fx = 0, fy = 0, cx = 0, cy = 0;
    float k1 = 0, k2 = 0, k3 = 0, p1 = 0, p2 = 0;
    float c2w[16];               // camera-to-world, OpenGL axes, row-major
};

struct LoadedScene {
    std::vector<LoadedCamera> cameras;
    std::vector<float> xyz;      // seed points
    std::vector<uint8_t> rgb;
};

// Detects the layout under `root` (transforms.json -> Nerfstudio;
// cameras.bin in root or sparse/0 -> COLMAP (text models too); keyframes/ or
// cameras.json -> Polycam) and reads cameras and seed points.  Cameras are
// sorted by file name as the reference does.  Throws on an unknown layout.
LoadedScene load_scene(const std::string &root, const std::string &colmap_image_dir = "");

// Points of a PLY file (x, y, z; red, green, blue when present).
void read_ply_points(const std::string &path, std::vector<float> &xyz, std::vector<uint8_t> &rgb);

}  // namespace io
}  // namespace msplat
