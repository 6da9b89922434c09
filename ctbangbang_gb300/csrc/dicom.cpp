// dicom.cpp -- the final slice stack as a DICOM CT image series.
//
// The reference writes the float32 stack as one raw file (finish_and_cleanup,
// src/setup.cu:769-787); its resources carry an example CT image
// (resources/testfile.dcm: CT Image Storage, explicit VR little endian, 16-bit
// signed pixels).  This writer produces one such file per final slice so that
// the stack opens in a DICOM viewer.  Encoding from the DICOM standard:
// PS3.10 file format (128-byte preamble, "DICM", file meta group 0002 in
// explicit VR little endian) and PS3.5 data elements (explicit VR: 2-byte
// length, or 2 reserved bytes and a 4-byte length for OB/OW; values padded to
// even length with NUL for UI and blanks otherwise; elements in tag order).
//
// Pixels: HU rounded to the nearest integer and clamped to int16, rescale
// slope 1, intercept 0.  Pixel (column i, row j) is the voxel centre the
// backprojector uses, x = pix (i - (nx-1)/2) + Xorigin, y likewise, with rows
// along +x and columns along +y; slice k lies at start + dir k SliceThickness
// as finalize places it.  UIDs are 2.25.<random 128-bit decimal> (PS3.5 B.2).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "ctbb_internal.h"

namespace ctbb {

namespace {

const char kCtImageStorage[] = "1.2.840.10008.5.1.4.1.1.2";
const char kExplicitVrLittleEndian[] = "1.2.840.10008.1.2.1";

std::string random_uid(std::mt19937_64 &rng)
{
    unsigned __int128 v = ((unsigned __int128)rng() << 64) | rng();
    char digits[48];
    int n = 0;
    do {
        digits[n++] = (char)('0' + (int)(v % 10));
        v /= 10;
    } while (v);
    std::string s = "2.25.";
    while (n) s += digits[--n];
    return s;
}

// DS: decimal string of at most 16 characters
std::string ds(double v)
{
    char buf[64];
    for (int prec = 10; prec >= 1; --prec) {
        snprintf(buf, sizeof(buf), "%.*g", prec, v);
        if (strlen(buf) <= 16) break;
    }
    return buf;
}

struct Writer {
    std::vector<uint8_t> out;
    void u16(uint16_t v) { out.push_back((uint8_t)v), out.push_back((uint8_t)(v >> 8)); }
    void u32(uint32_t v) { u16((uint16_t)v), u16((uint16_t)(v >> 16)); }
    void raw(const void *p, size_t n)
    {
        const uint8_t *b = static_cast<const uint8_t *>(p);
        out.insert(out.end(), b, b + n);
    }
    // element with a 2-byte length (every VR here except OB / OW)
    void elem(uint16_t group, uint16_t element, const char vr[2], const std::string &value)
    {
        std::string v = value;
        if (v.size() & 1) v += (vr[0] == 'U' && vr[1] == 'I') ? '\0' : ' ';
        u16(group), u16(element), raw(vr, 2), u16((uint16_t)v.size()), raw(v.data(), v.size());
    }
    void us(uint16_t group, uint16_t element, uint16_t value)
    {
        u16(group), u16(element), raw("US", 2), u16(2), u16(value);
    }
    // OB / OW: 2 reserved bytes, 4-byte length (even)
    void long_elem(uint16_t group, uint16_t element, const char vr[2], const void *p, uint32_t n)
    {
        u16(group), u16(element), raw(vr, 2), u16(0), u32(n), raw(p, n);
    }
};

}  // namespace

}  // namespace ctbb

using namespace ctbb;

extern "C" int ctbb_write_dicom_series(const struct recon_metadata *mr, const float *h_stack, int n_slices,
                                       float mu_water, const char *out_dir)
{
    clear_error();
    if (!mr || !h_stack || !out_dir || n_slices <= 0 || !(mu_water >= 0.0f)) {
        set_error("ctbb_write_dicom_series: bad argument");
        return CTBB_ERR_ARGUMENT;
    }
    const struct recon_params &rp = mr->rp;
    if (rp.nx == 0 || rp.ny == 0 || rp.nx > 65535 || rp.ny > 65535 || !(rp.slice_thickness > 0.0f)) {
        set_error("ctbb_write_dicom_series: image %u x %u / slice thickness %g not writable", rp.nx, rp.ny,
                  (double)rp.slice_thickness);
        return CTBB_ERR_ARGUMENT;
    }
    std::random_device rd;
    std::mt19937_64 rng(((uint64_t)rd() << 32) ^ rd());
    const std::string study = random_uid(rng), series = random_uid(rng), frame_of_ref = random_uid(rng);
    const double pix_x = (double)rp.recon_fov / rp.nx, pix_y = (double)rp.recon_fov / rp.ny;
    const double x0 = pix_x * (0.0 - (rp.nx - 1) / 2.0) + rp.x_origin;
    const double y0 = pix_y * (0.0 - (rp.ny - 1) / 2.0) + rp.y_origin;
    const int dir = recon_direction_of(rp);
    std::string stem = rp.output_file[0] ? std::string(rp.output_file) : std::string("slice");
    size_t dot = stem.find_last_of('.');
    if (dot != std::string::npos && dot > 0) stem.resize(dot);
    const size_t plane = (size_t)rp.nx * rp.ny;
    std::vector<int16_t> pix(plane);
    char kernel[32];
    snprintf(kernel, sizeof(kernel), "%d", rp.recon_kernel);
    for (int k = 0; k < n_slices; ++k) {
        const float *src = h_stack + (size_t)k * plane;
        for (size_t e = 0; e < plane; ++e) {
            double hu = mu_water > 0.0f ? 1000.0 * ((double)src[e] - mu_water) / mu_water : (double)src[e];
            double r = std::nearbyint(hu);
            if (!(r >= -32768.0)) r = -32768.0;  // NaN too
            if (r > 32767.0) r = 32767.0;
            pix[e] = (int16_t)r;
        }
        const float z = rp.start_pos + (float)(dir * k) * rp.slice_thickness;
        const std::string sop = series + "." + std::to_string(k + 1);
        Writer meta;
        meta.long_elem(0x0002, 0x0001, "OB", "\x00\x01", 2);
        meta.elem(0x0002, 0x0002, "UI", kCtImageStorage);
        meta.elem(0x0002, 0x0003, "UI", sop);
        meta.elem(0x0002, 0x0010, "UI", kExplicitVrLittleEndian);
        meta.elem(0x0002, 0x0012, "UI", "2.25.316125587360742918112963302519612771862");
        meta.elem(0x0002, 0x0013, "SH", "CTBB_GB300");
        Writer f;
        f.out.assign(128, 0);
        f.raw("DICM", 4);
        f.u16(0x0002), f.u16(0x0000), f.raw("UL", 2), f.u16(4), f.u32((uint32_t)meta.out.size());
        f.raw(meta.out.data(), meta.out.size());
        f.elem(0x0008, 0x0005, "CS", "ISO_IR 100");
        f.elem(0x0008, 0x0008, "CS", "DERIVED\\PRIMARY\\AXIAL");
        f.elem(0x0008, 0x0016, "UI", kCtImageStorage);
        f.elem(0x0008, 0x0018, "UI", sop);
        f.elem(0x0008, 0x0060, "CS", "CT");
        f.elem(0x0008, 0x103E, "LO", "wFBP ctbangbang_gb300");
        f.elem(0x0010, 0x0010, "PN", "");
        f.elem(0x0010, 0x0020, "LO", "");
        f.elem(0x0018, 0x0050, "DS", ds(rp.slice_thickness));
        f.elem(0x0018, 0x1100, "DS", ds(rp.recon_fov));
        f.elem(0x0018, 0x1110, "DS", ds(mr->cg.src_to_det));
        f.elem(0x0018, 0x1111, "DS", ds(mr->cg.r_f));
        f.elem(0x0018, 0x1210, "SH", kernel);
        f.elem(0x0020, 0x000D, "UI", study);
        f.elem(0x0020, 0x000E, "UI", series);
        f.elem(0x0020, 0x0011, "IS", "1");
        f.elem(0x0020, 0x0013, "IS", std::to_string(k + 1));
        f.elem(0x0020, 0x0032, "DS", ds(x0) + "\\" + ds(y0) + "\\" + ds(z));
        f.elem(0x0020, 0x0037, "DS", "1\\0\\0\\0\\1\\0");
        f.elem(0x0020, 0x0052, "UI", frame_of_ref);
        f.elem(0x0020, 0x1041, "DS", ds(z));
        f.us(0x0028, 0x0002, 1);
        f.elem(0x0028, 0x0004, "CS", "MONOCHROME2");
        f.us(0x0028, 0x0010, (uint16_t)rp.ny);
        f.us(0x0028, 0x0011, (uint16_t)rp.nx);
        f.elem(0x0028, 0x0030, "DS", ds(pix_y) + "\\" + ds(pix_x));
        f.us(0x0028, 0x0100, 16);
        f.us(0x0028, 0x0101, 16);
        f.us(0x0028, 0x0102, 15);
        f.us(0x0028, 0x0103, 1);
        f.elem(0x0028, 0x1050, "DS", "40");
        f.elem(0x0028, 0x1051, "DS", "400");
        f.elem(0x0028, 0x1052, "DS", "0");
        f.elem(0x0028, 0x1053, "DS", "1");
        f.elem(0x0028, 0x1054, "LO", "HU");
        // pixels little endian whatever the host order
        std::vector<uint8_t> bytes(plane * 2);
        for (size_t e = 0; e < plane; ++e) {
            uint16_t u = (uint16_t)pix[e];
            bytes[2 * e] = (uint8_t)u;
            bytes[2 * e + 1] = (uint8_t)(u >> 8);
        }
        f.long_elem(0x7FE0, 0x0010, "OW", bytes.data(), (uint32_t)bytes.size());
        char path[4096 + 512];
        snprintf(path, sizeof(path), "%s/%s_%04d.dcm", out_dir, stem.c_str(), k + 1);
        FILE *fp = fopen(path, "wb");
        if (!fp) {
            set_error("ctbb_write_dicom_series: cannot create %s", path);
            return CTBB_ERR_IO;
        }
        size_t wrote = fwrite(f.out.data(), 1, f.out.size(), fp);
        int closed = fclose(fp);
        if (wrote != f.out.size() || closed != 0) {
            set_error("ctbb_write_dicom_series: short write to %s", path);
            return CTBB_ERR_IO;
        }
    }
    return CTBB_OK;
}
