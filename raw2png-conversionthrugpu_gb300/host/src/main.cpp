// main.cpp -- gpu_png_encoder, the command line of the reference
// (src/main.cpp:1-257) on the GB300 encoder.
//
//   gpu_png_encoder <input.dcm> <output.png> [options]     single file
//   gpu_png_encoder <input.dcm> <output_dir> --all          every frame
//   gpu_png_encoder <input_dir> <output_dir> [options]      folder batch
//   gpu_png_encoder --bench-deflate [N]                     GPU DEFLATE benchmark
//   gpu_png_encoder <input.dcm> --probe                     print the parsed header (no GPU)
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <string>
#include <vector>

#include "batch_processor.h"
#include "dicom_loader.h"
#include "file_type.h"
#include "parallel_deflate.h"
#include "pipeline.h"

static void usage(const char* prog)
{
    std::fprintf(stderr,
                 "Usage: %s <input> <output> [options]\n"
                 "  <input>  : DICOM file (uncompressed Implicit/Explicit VR Little Endian), an\n"
                 "             uncompressed TIFF (.tif/.tiff), or a folder\n"
                 "  <output> : a .png file, or a folder with --all / folder input\n"
                 "  --all                every frame as <output>/slice_NNNN.png   (alias: -all)\n"
                 "  --frame N            export DICOM frame N (0-based)\n"
                 "  --strip-height N     rows per strip (default 1024)\n"
                 "  --level N            0 = stored, 1 = LZ77 + fixed Huffman, 2-9 = dynamic\n"
                 "                       Huffman over a run-length parse (default 3)\n"
                 "  --threads N          accepted; DEFLATE runs on the GPU\n"
                 "  --verbose            per-file report\n"
                 "  --batch-workers N    folder mode file readers (default: auto)\n"
                 "  --batch-verbose      per-file wall time in folder mode\n"
                 "  --gpu-streams N      frames in flight for --all (default 4)\n"
                 "  --gpu-deflate, --gpu-lz77, --no-gpu-lz77, --gpu-lz77-debug   accepted (always GPU)\n"
                 "  --format png|bmp     output format (default png); bmp: uncompressed 8-bit gray /\n"
                 "                       24-bit BGR, written on the GPU\n"
                 "  --strip-pipeline     run strips through gpu_filter + GpuDeflateBackend\n"
                 "  --idat-chunk N       IDAT chunks of at most N bytes (default: one IDAT)\n"
                 "  --device N           GPU ordinal\n"
                 "  --probe              print the parsed DICOM/TIFF header as JSON and exit\n"
                 "  --bench-deflate [N]  GPU DEFLATE benchmark on N bytes (default 2400000)\n",
                 prog);
}

static int probe(const char* path)
{
    if (is_tiff_file(path)) {
        TiffSource t;
        if (!t.open(path)) return 1;
        const ImageInfo& i = t.info();
        std::vector<uint8_t> buf((size_t)i.width * i.bpp * 64);
        uint64_t sum = 0;
        int rows = 0, n;
        while ((n = t.read_strip(buf.data(), 64)) > 0) {       // reads every strip
            for (size_t k = 0; k < (size_t)n * i.width * i.bpp; k++) sum += buf[k];
            rows += n;
        }
        std::printf("{\"format\": \"tiff\", \"width\": %u, \"height\": %u, \"channels\": %d, "
                    "\"bits_per_sample\": %d, \"bpp\": %d, \"rows_read\": %d, \"byte_sum\": %llu}\n",
                    i.width, i.height, i.channels, i.bits_per_sample, i.bpp, rows, (unsigned long long)sum);
        return rows == (int)i.height ? 0 : 1;
    }
    DicomSource s;
    if (!s.open(path)) return 1;
    const ImageInfo& i = s.info();
    const DicomPixelParams& p = *s.dicom_params();
    std::printf("{\"transfer_syntax\": \"%s\", \"photometric\": \"%s\", \"width\": %u, \"height\": %u, "
                "\"channels\": %d, \"bits_per_sample\": %d, \"bpp\": %d, \"frames\": %d, "
                "\"bits_allocated\": %d, \"bits_stored\": %d, \"high_bit\": %d, \"pixel_rep\": %d, "
                "\"apply_rescale\": %d, \"rescale_slope\": %.9g, \"rescale_intercept\": %.9g, "
                "\"apply_window\": %d, \"window_center\": %.9g, \"window_width\": %.9g}\n",
                s.transfer_syntax_.c_str(), s.photometric_.c_str(), i.width, i.height, i.channels, i.bits_per_sample,
                i.bpp, s.num_frames(), p.bits_allocated, p.bits_stored, p.high_bit, p.pixel_rep, p.apply_rescale,
                (double)p.rescale_slope, (double)p.rescale_intercept, p.apply_window, (double)p.window_center,
                (double)p.window_width);
    for (int f = 0; f < s.num_frames(); f++)
        if (!s.load_frame(f)) return 1;
    return 0;
}

int main(int argc, char* argv[])
{
    for (int i = 1; i < argc; i++) {
        if (std::strcmp(argv[i], "--bench-deflate") == 0) {
            size_t n = 2400000;
            if (i + 1 < argc && std::isdigit((unsigned char)argv[i + 1][0])) n = std::strtoull(argv[i + 1], nullptr, 10);
            bench_deflate(n, 1);
            return 0;
        }
    }
    if (argc >= 3 && std::strcmp(argv[2], "--probe") == 0) return probe(argv[1]);
    if (argc < 3) {
        usage(argv[0]);
        return 1;
    }
    const char* input = argv[1];
    const char* output = argv[2];
    PipelineConfig cfg;
    BatchConfig bcfg;
    bool all_frames = false;
    for (int i = 3; i < argc; i++) {
        const char* a = argv[i];
        const bool has = i + 1 < argc;
        if (!std::strcmp(a, "--strip-height") && has) cfg.strip_height = std::atoi(argv[++i]);
        else if (!std::strcmp(a, "--threads") && has) cfg.deflate_threads = std::atoi(argv[++i]);
        else if (!std::strcmp(a, "--level") && has) cfg.deflate_level = std::atoi(argv[++i]);
        else if (!std::strcmp(a, "--frame") && has) cfg.frame = std::atoi(argv[++i]);
        else if (!std::strcmp(a, "--all") || !std::strcmp(a, "-all")) all_frames = true;
        else if (!std::strcmp(a, "--verbose")) cfg.verbose = true;
        else if (!std::strcmp(a, "--batch-workers") && has) bcfg.num_workers = std::atoi(argv[++i]);
        else if (!std::strcmp(a, "--batch-verbose")) bcfg.batch_verbose = true;
        else if (!std::strcmp(a, "--gpu-streams") && has) cfg.gpu_streams = std::atoi(argv[++i]);
        else if (!std::strcmp(a, "--gpu-deflate") || !std::strcmp(a, "--gpu-lz77") || !std::strcmp(a, "--no-gpu-lz77") ||
                 !std::strcmp(a, "--gpu-lz77-debug")) {
        } else if (!std::strcmp(a, "--strip-pipeline")) cfg.strip_pipeline = true;
        else if (!std::strcmp(a, "--idat-chunk") && has) cfg.idat_chunk = std::atoi(argv[++i]);
        else if (!std::strcmp(a, "--device") && has) cfg.device = std::atoi(argv[++i]);
        else if (!std::strcmp(a, "--format") && has) {
            const char* f = argv[++i];
            if (!std::strcmp(f, "png") || !std::strcmp(f, "PNG")) cfg.format = ExportFormat::PNG;
            else if (!std::strcmp(f, "bmp") || !std::strcmp(f, "BMP")) cfg.format = ExportFormat::BMP;
            else {
                std::fprintf(stderr, "Unknown format '%s'. Supported: png, bmp\n", f);
                return 1;
            }
        } else {
            std::fprintf(stderr, "Unknown option: %s\n", a);
            usage(argv[0]);
            return 1;
        }
    }
    if (cfg.deflate_level < 0) cfg.deflate_level = 0;
    if (cfg.deflate_level > 9) cfg.deflate_level = 9;
    if (cfg.strip_height < 0) cfg.strip_height = 0;
    const bool use_bmp = cfg.format == ExportFormat::BMP;
    if (all_frames && use_bmp) {      // src/main.cpp:210-214
        std::fprintf(stderr, "Note: --all applies only to DICOM PNG mode; ignoring.\n");
        all_frames = false;
    }
    std::error_code ec;
    if (std::filesystem::is_directory(input, ec)) {
        if (!encode_folder(input, output, cfg, bcfg)) {
            std::fprintf(stderr, "Batch encoding finished with errors.\n");
            return 1;
        }
        return 0;
    }
    bool good;
    if (use_bmp) good = is_tiff_file(input)  ? encode_tiff_to_bmp(input, output, cfg)
                      : is_raw_file(input)   ? encode_raw_to_bmp(input, output, cfg)
                                             : encode_dicom_to_bmp(input, output, cfg);
    else if (is_tiff_file(input)) good = encode_tiff_to_png(input, output, cfg);
    else if (is_raw_file(input)) good = encode_raw_to_png(input, output, cfg);
    else if (all_frames) good = encode_dicom_all_frames_to_png(input, output, cfg);
    else good = encode_dicom_to_png(input, output, cfg);
    if (!good) {
        std::fprintf(stderr, "Encoding failed.\n");
        return 1;
    }
    if (cfg.verbose && !all_frames) std::printf("Done -> %s\n", output);
    return 0;
}
