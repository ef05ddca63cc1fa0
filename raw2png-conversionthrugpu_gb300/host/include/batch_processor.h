#pragma once
// Folder batch mode (the reference's include/batch_processor.h:15-48) on the
// continuous-batching server: every DICOM and TIFF file of a folder (top
// level) is submitted as it is read, and written as <stem>.png; multi-frame
// DICOM files go to <stem>/slice_NNNN.png.  16-bit grayscale frames become 8-bit PNGs through
// the folder batch's windowing (Q15 map when eligible, else the FP32 table,
// src/batch_processor.cpp:397-409); other frames keep their depth with the
// DICOM window transform.
#include "pipeline.h"

struct BatchConfig {
    int  num_workers   = 0;      // file readers; 0 = auto
    bool batch_verbose = false;
};

bool encode_folder(const char* input_dir, const char* output_dir, const PipelineConfig& cfg,
                   const BatchConfig& batch_cfg);
