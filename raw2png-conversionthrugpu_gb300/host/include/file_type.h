#pragma once
// Input format detection (the reference's include/file_type.h:7-18).
bool ends_with_ci(const char* s, const char* suffix);
bool is_tiff_file(const char* path);
bool is_raw_file(const char* path);
bool is_dicom_file(const char* path);   // DICOM extension, or "DICM" at byte 128
