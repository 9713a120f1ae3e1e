// A caller of the reference's C++ interface (am::morph, morph.h:9-145), built
// against include/atomorph_gb300.hpp and linked with the GB300 library: key
// frames in with add_pixel, the pipeline stepped the way the reference's demo
// steps it (iterate, wait while busy, synchronize; demo/main.cpp:220-260), a
// few refinement steps, then whole frames (get_pixels(t)), the pixel list of
// every blob of one key frame (get_pixels(blob, t)) and get_blob.
//
//   morph_roundtrip <in.bin> <out_dir>
//   in.bin: uint32 K, W, H, then K frames of W * H RGBA8 pixels.
// Writes out_dir/chains.bin (uint64 K, C, N, widths[C], points[K * N],
// int32 order[K * C]), frame_<i>.bin (W * H * 4 bytes at times kTimes[i]),
// blobs.bin (uint64 count, then per blob: uint64 n, n x (x, y) uint16,
// n x RGBA8, uint64 surface size, uint64 group) and state.txt.
#include <chrono>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

#include "atomorph_gb300.hpp"

static const double kTimes[3] = {0.1, 0.45, 0.8};

static void wait_idle(am::morph &m) {
    while (m.is_busy()) std::this_thread::sleep_for(std::chrono::microseconds(200));
}

int main(int argc, char **argv) {
    if (argc != 3) return 2;
    FILE *in = std::fopen(argv[1], "rb");
    if (!in) return 3;
    uint32_t hdr[3];
    if (std::fread(hdr, 4, 3, in) != 3) return 3;
    const uint32_t K = hdr[0], W = hdr[1], H = hdr[2];
    std::vector<uint8_t> img((size_t)K * W * H * 4);
    if (std::fread(img.data(), 1, img.size(), in) != img.size()) return 3;
    std::fclose(in);
    const std::string dir = argv[2];

    am::morph m;
    m.set_seed(7);
    m.set_blob_delimiter(am::HSP);
    m.set_motion(am::SPLINE);
    m.set_fading(am::PERLIN);
    for (uint32_t k = 0; k < K; ++k)
        for (uint32_t y = 0; y < H; ++y)
            for (uint32_t x = 0; x < W; ++x) {
                const uint8_t *p = &img[(((size_t)k * H + y) * W + x) * 4];
                if (p[3] > 0 && !m.add_pixel(k, am::create_pixel((uint16_t)x, (uint16_t)y, p[0], p[1], p[2], p[3])))
                    return 4;
            }
    m.set_resolution((uint16_t)W, (uint16_t)H);
    m.synchronize();
    for (int i = 0; i < 100000 && m.get_state() < am::STATE_ATOM_MORPHING; ++i) {
        m.iterate(1);
        wait_idle(m);
        m.synchronize();
    }
    if (m.get_state() != am::STATE_ATOM_MORPHING) return 5;
    m.iterate(20);
    wait_idle(m);
    if (!m.synchronize()) return 6;

    am_morph *h = m.handle();
    const uint64_t C = am_get_chain_count(h), N = am_get_atom_count(h), KK = am_get_frame_count(h);
    std::vector<uint64_t> widths(C), pts(KK * N);
    std::vector<int32_t> order(KK * C);
    if (am_export_chains(h, widths.data(), pts.data(), order.data()) != AM_OK) return 7;
    FILE *f = std::fopen((dir + "/chains.bin").c_str(), "wb");
    const uint64_t sizes[3] = {KK, C, N};
    std::fwrite(sizes, 8, 3, f);
    std::fwrite(widths.data(), 8, C, f);
    std::fwrite(pts.data(), 8, pts.size(), f);
    std::fwrite(order.data(), 4, order.size(), f);
    std::fclose(f);

    std::vector<am::pixel> frame;
    for (int i = 0; i < 3; ++i) {
        m.get_pixels(kTimes[i], &frame);
        if (frame.size() != (size_t)W * H) return 8;
        FILE *o = std::fopen((dir + "/frame_" + std::to_string(i) + ".bin").c_str(), "wb");
        for (const am::pixel &p : frame) std::fwrite(&p.c, 1, 4, o);
        std::fclose(o);
    }

    const double t = kTimes[1];
    const size_t key = m.get_frame_key(t), nb = m.get_blob_count(key);
    FILE *o = std::fopen((dir + "/blobs.bin").c_str(), "wb");
    const uint64_t count = nb;
    std::fwrite(&count, 8, 1, o);
    for (size_t b = 0; b < nb; ++b) {
        std::vector<am::pixel> px;
        const am::blob *bl = m.get_pixels(b, t, &px);
        if (!bl || bl != m.get_blob(key, b) || bl->index != b) return 9;
        const uint64_t n = px.size(), surface = bl->surface.size(), group = bl->group;
        std::fwrite(&n, 8, 1, o);
        for (const am::pixel &p : px) std::fwrite(&p.x, 2, 2, o);
        for (const am::pixel &p : px) std::fwrite(&p.c, 1, 4, o);
        std::fwrite(&surface, 8, 1, o);
        std::fwrite(&group, 8, 1, o);
    }
    std::fclose(o);
    if (m.get_pixels(nb, t, &frame) != nullptr || m.get_blob(key, nb) != nullptr) return 10;
    FILE *s = std::fopen((dir + "/state.txt").c_str(), "w");
    std::fprintf(s, "%u %.17g\n", m.get_state(), m.get_energy());
    std::fclose(s);
    return 0;
}
