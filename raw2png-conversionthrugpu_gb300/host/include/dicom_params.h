#pragma once
// DICOM pixel transform parameters handed from a DICOM source to the GPU
// window stage.  Members, order and defaults are those of the reference's
// DicomPixelParams (include/dicom_params.h:6-21) so callers compile
// unchanged; the layout is also that of r2p_dicom_params in r2p.h.
// A null DicomPixelParams* means "no DICOM transform".
struct DicomPixelParams {
    int   bits_allocated    = 16;      // (0028,0100)
    int   bits_stored       = 16;      // (0028,0101)
    int   high_bit          = 15;      // (0028,0102); right-align shift = high_bit - bits_stored + 1
    int   pixel_rep         = 0;       // (0028,0103) 0 unsigned, 1 two's complement
    int   apply_rescale     = 0;       // slope/intercept present and not the identity
    float rescale_slope     = 1.f;     // (0028,1053)
    float rescale_intercept = 0.f;     // (0028,1052)
    int   apply_window      = 0;       // window centre and width present, width > 0
    float window_center     = 32768.f; // (0028,1050)
    float window_width      = 65536.f; // (0028,1051)
};
