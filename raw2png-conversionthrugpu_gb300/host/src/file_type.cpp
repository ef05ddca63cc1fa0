// file_type.cpp -- input format detection (src/file_type.cpp of the reference:
// extensions, and the Part-10 "DICM" magic at byte 128).
#include "file_type.h"

#include <cctype>
#include <cstdio>
#include <cstring>

bool ends_with_ci(const char* s, const char* suffix)
{
    const size_t a = std::strlen(s), b = std::strlen(suffix);
    if (a < b) return false;
    for (size_t i = 0; i < b; i++)
        if (std::tolower((unsigned char)s[a - b + i]) != std::tolower((unsigned char)suffix[i])) return false;
    return true;
}

bool is_tiff_file(const char* path)
{
    return ends_with_ci(path, ".tif") || ends_with_ci(path, ".tiff");
}

bool is_raw_file(const char* path)
{
    static const char* ext[] = {".cr2", ".nef", ".dng", ".arw", ".raw", ".raf", ".orf", ".rw2"};
    for (const char* e : ext)
        if (ends_with_ci(path, e)) return true;
    return false;
}

bool is_dicom_file(const char* path)
{
    static const char* ext[] = {".dcm", ".dicom", ".dic", ".ima"};
    for (const char* e : ext)
        if (ends_with_ci(path, e)) return true;
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    char m[4] = {0, 0, 0, 0};
    const bool got = std::fseek(f, 128, SEEK_SET) == 0 && std::fread(m, 1, 4, f) == 4;
    std::fclose(f);
    return got && std::memcmp(m, "DICM", 4) == 0;
}
