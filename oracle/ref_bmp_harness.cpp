// ref_bmp_harness.cpp -- TEST INFRASTRUCTURE.
//
// Compiles the reference's pipeline translation unit (src/pipeline.cpp) and
// its BMP writer (src/bmp_writer.cpp), both included unchanged from the
// reference tree through the include path that oracle/build_oracle.py sets,
// and runs the reference's own encode_source_to_bmp (src/pipeline.cpp:2057-2060
// -> run_bmp_from_source :1944-2004) on an in-memory image source, so the
// tests can pin the BMP export against files the reference itself wrote.
//
// The executable is linked with unresolved symbols ignored: the GPU, decoder
// and PNG code that the translation unit references is never reached from
// the BMP path.
//
// usage: ref_bmp_runner in.raw out.bmp width height channels bits_per_sample
//        dicom(0|1) bits_allocated bits_stored high_bit pixel_rep
//        apply_rescale slope intercept apply_window center width
// (floats as C99 hex literals, so they pass through exactly)
#include "pipeline.cpp"
#include "bmp_writer.cpp"

#include <cstdlib>

namespace {

struct MemSource : ImageSource {
    ImageInfo inf;
    DicomPixelParams dp;
    bool dicom = false;
    std::vector<uint8_t> px;
    uint32_t next = 0;

    const ImageInfo& info() const override { return inf; }
    const DicomPixelParams* dicom_params() const override { return dicom ? &dp : nullptr; }
    int read_strip(uint8_t* out, int max_rows) override
    {
        const uint32_t rows = std::min<uint32_t>((uint32_t)max_rows, inf.height - next);
        const size_t rb = (size_t)inf.width * inf.bpp;
        std::memcpy(out, px.data() + (size_t)next * rb, rows * rb);
        next += rows;
        return (int)rows;
    }
};

}  // namespace

int main(int argc, char** argv)
{
    if (argc != 18) {
        std::fprintf(stderr, "ref_bmp_runner: expected 17 arguments\n");
        return 2;
    }
    MemSource src;
    src.inf.width = (uint32_t)std::atoi(argv[3]);
    src.inf.height = (uint32_t)std::atoi(argv[4]);
    src.inf.channels = std::atoi(argv[5]);
    src.inf.bits_per_sample = std::atoi(argv[6]);
    src.inf.bpp = src.inf.channels * src.inf.bits_per_sample / 8;
    src.dicom = std::atoi(argv[7]) != 0;
    src.dp.bits_allocated = std::atoi(argv[8]);
    src.dp.bits_stored = std::atoi(argv[9]);
    src.dp.high_bit = std::atoi(argv[10]);
    src.dp.pixel_rep = std::atoi(argv[11]);
    src.dp.apply_rescale = std::atoi(argv[12]) != 0;
    src.dp.rescale_slope = std::strtof(argv[13], nullptr);
    src.dp.rescale_intercept = std::strtof(argv[14], nullptr);
    src.dp.apply_window = std::atoi(argv[15]) != 0;
    src.dp.window_center = std::strtof(argv[16], nullptr);
    src.dp.window_width = std::strtof(argv[17], nullptr);
    const size_t n = (size_t)src.inf.width * src.inf.height * src.inf.bpp;
    src.px.resize(n);
    FILE* f = std::fopen(argv[1], "rb");
    if (!f || std::fread(src.px.data(), 1, n, f) != n) {
        std::fprintf(stderr, "ref_bmp_runner: cannot read %s\n", argv[1]);
        return 2;
    }
    std::fclose(f);
    return encode_source_to_bmp(src, argv[2]) ? 0 : 1;
}
