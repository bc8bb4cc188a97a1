// Micro-CT slice loading: a self-contained PNG decoder (zlib/DEFLATE per RFC 1950/1951, PNG
// filters per the PNG specification) and the uct-config file naming of the reference
// (ConfigFiles/uct_config.cpp:150-198: DIR_PATH + FILENAME + zero-padded index + EXTENSION, or the
// first SLICES lines of IMG_FILES_LIST).
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>

#include "sequences.h"

namespace rwnmr_host
{
namespace
{
// ---- DEFLATE --------------------------------------------------------------------------------
struct Bits
{
    const uint8_t *p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;
    bool bad = false;
    int need(int k)
    {
        while (cnt < k)
        {
            if (pos >= n)
            {
                bad = true;
                return 0;
            }
            buf |= (uint32_t)p[pos++] << cnt;
            cnt += 8;
        }
        int v = (int)(buf & ((1u << k) - 1));
        buf >>= k;
        cnt -= k;
        return v;
    }
};

// Canonical Huffman table: count of codes per length and the symbols in code order.
struct Huff
{
    uint16_t count[16] = {0};
    uint16_t sym[320] = {0};
    bool build(const uint8_t *len, int n)
    {
        std::memset(count, 0, sizeof count);
        for (int s = 0; s < n; s++) count[len[s]]++;
        count[0] = 0;
        uint16_t offs[16];
        offs[1] = 0;
        for (int l = 1; l < 15; l++) offs[l + 1] = offs[l] + count[l];
        for (int s = 0; s < n; s++)
            if (len[s]) sym[offs[len[s]]++] = (uint16_t)s;
        return true;
    }
    int decode(Bits &b) const
    {
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; l++)
        {
            code |= b.need(1);
            if (b.bad) return -1;
            const int c = count[l];
            if (code - c < first) return sym[index + (code - first)];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        return -1;
    }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_block(Bits &b, const Huff &lit, const Huff &dist, std::vector<uint8_t> &out)
{
    for (;;)
    {
        int s = lit.decode(b);
        if (s < 0) return false;
        if (s < 256) out.push_back((uint8_t)s);
        else if (s == 256) return true;
        else
        {
            s -= 257;
            if (s >= 29) return false;
            int len = kLenBase[s] + b.need(kLenExtra[s]);
            int d = dist.decode(b);
            if (d < 0 || d >= 30) return false;
            size_t back = kDistBase[d] + b.need(kDistExtra[d]);
            if (b.bad || back > out.size()) return false;
            size_t from = out.size() - back;
            for (int k = 0; k < len; k++) out.push_back(out[from + k]);
        }
    }
}

bool inflate(const uint8_t *src, size_t n, std::vector<uint8_t> &out)
{
    Bits b{src, n};
    int last;
    do
    {
        last = b.need(1);
        int type = b.need(2);
        if (b.bad) return false;
        if (type == 0)
        {
            b.buf = 0;
            b.cnt = 0; // stored block: skip to the byte boundary
            if (b.pos + 4 > n) return false;
            unsigned len = src[b.pos] | (src[b.pos + 1] << 8);
            b.pos += 4;
            if (b.pos + len > n) return false;
            out.insert(out.end(), src + b.pos, src + b.pos + len);
            b.pos += len;
        }
        else if (type == 1)
        {
            uint8_t l[288], d[30];
            for (int i = 0; i < 144; i++) l[i] = 8;
            for (int i = 144; i < 256; i++) l[i] = 9;
            for (int i = 256; i < 280; i++) l[i] = 7;
            for (int i = 280; i < 288; i++) l[i] = 8;
            for (int i = 0; i < 30; i++) d[i] = 5;
            Huff hl, hd;
            hl.build(l, 288);
            hd.build(d, 30);
            if (!inflate_block(b, hl, hd, out)) return false;
        }
        else if (type == 2)
        {
            const int nlen = b.need(5) + 257, ndist = b.need(5) + 1, ncode = b.need(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (int i = 0; i < ncode; i++) cl[order[i]] = (uint8_t)b.need(3);
            Huff hc;
            hc.build(cl, 19);
            uint8_t lens[320] = {0};
            int idx = 0;
            while (idx < nlen + ndist)
            {
                int s = hc.decode(b);
                if (s < 0) return false;
                if (s < 16) lens[idx++] = (uint8_t)s;
                else
                {
                    int rep, val = 0;
                    if (s == 16)
                    {
                        if (idx == 0) return false;
                        val = lens[idx - 1];
                        rep = 3 + b.need(2);
                    }
                    else if (s == 17) rep = 3 + b.need(3);
                    else rep = 11 + b.need(7);
                    if (idx + rep > nlen + ndist) return false;
                    while (rep--) lens[idx++] = (uint8_t)val;
                }
            }
            Huff hl, hd;
            hl.build(lens, nlen);
            hd.build(lens + nlen, ndist);
            if (!inflate_block(b, hl, hd, out)) return false;
        }
        else
            return false;
        if (b.bad) return false;
    } while (!last);
    return true;
}

uint32_t be32(const uint8_t *p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

int paeth(int a, int b, int c)
{
    int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc) return a;
    return pb <= pc ? b : c;
}
} // namespace

bool png_solid_mask(const std::string &path, int &width, int &height, std::vector<uint8_t> &mask, std::string &err)
{
    std::ifstream f(path, std::ios::binary);
    if (!f)
    {
        err = "Error: No image data in file " + path;
        return false;
    }
    std::vector<uint8_t> data((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (data.size() < 8 || std::memcmp(data.data(), sig, 8) != 0)
    {
        err = path + ": not a PNG file";
        return false;
    }
    int depth = 0, ctype = 0, interlace = 0;
    std::vector<uint8_t> idat, pal;
    size_t p = 8;
    while (p + 12 <= data.size())
    {
        const uint32_t len = be32(&data[p]);
        const char *type = (const char *)&data[p + 4];
        if (p + 12 + len > data.size()) break;
        const uint8_t *d = &data[p + 8];
        if (!std::memcmp(type, "IHDR", 4) && len >= 13)
        {
            width = (int)be32(d);
            height = (int)be32(d + 4);
            depth = d[8];
            ctype = d[9];
            interlace = d[12];
        }
        else if (!std::memcmp(type, "PLTE", 4)) pal.assign(d, d + len);
        else if (!std::memcmp(type, "IDAT", 4)) idat.insert(idat.end(), d, d + len);
        else if (!std::memcmp(type, "IEND", 4)) break;
        p += 12 + len;
    }
    if (width <= 0 || height <= 0 || idat.size() < 2)
    {
        err = path + ": malformed PNG";
        return false;
    }
    if (interlace)
    {
        err = path + ": interlaced PNGs are not supported";
        return false;
    }
    const int chans = ctype == 0 ? 1 : ctype == 2 ? 3 : ctype == 3 ? 1 : ctype == 4 ? 2 : ctype == 6 ? 4 : 0;
    if (!chans || !(depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16))
    {
        err = path + ": unsupported PNG colour type / depth";
        return false;
    }
    std::vector<uint8_t> raw;
    if (!inflate(idat.data() + 2, idat.size() - 2, raw))
    {
        err = path + ": corrupt compressed data";
        return false;
    }
    const size_t bpp_bits = (size_t)chans * depth;
    const size_t stride = ((size_t)width * bpp_bits + 7) / 8;
    const size_t bpp = std::max<size_t>(1, bpp_bits / 8);
    if (raw.size() < (size_t)height * (stride + 1))
    {
        err = path + ": truncated image data";
        return false;
    }
    std::vector<uint8_t> prev(stride, 0), cur(stride);
    mask.assign((size_t)width * height, 0);
    for (int y = 0; y < height; y++)
    {
        const uint8_t *row = &raw[(size_t)y * (stride + 1)];
        const int ft = row[0];
        for (size_t i = 0; i < stride; i++)
        {
            const int a = i >= bpp ? cur[i - bpp] : 0, b = prev[i], c = i >= bpp ? prev[i - bpp] : 0;
            int v = row[1 + i];
            switch (ft)
            {
            case 1: v += a; break;
            case 2: v += b; break;
            case 3: v += (a + b) / 2; break;
            case 4: v += paeth(a, b, c); break;
            default: break;
            }
            cur[i] = (uint8_t)v;
        }
        for (int x = 0; x < width; x++)
        {
            // colour channels as an 8-bit image loader sees them (16-bit samples keep their high
            // byte, alpha is dropped); any non-zero channel is solid
            bool solid = false;
            if (depth < 8)
            {
                const size_t bit = (size_t)x * depth;
                const int v = (cur[bit / 8] >> (8 - depth - (bit % 8))) & ((1 << depth) - 1);
                if (ctype == 3) solid = (size_t)v * 3 + 2 < pal.size() && (pal[v * 3] | pal[v * 3 + 1] | pal[v * 3 + 2]);
                else solid = (v * 255 / ((1 << depth) - 1)) != 0;
            }
            else
            {
                const size_t px = (size_t)x * chans * (depth / 8);
                auto sample = [&](int ch) { return cur[px + (size_t)ch * (depth / 8)]; };
                if (ctype == 3)
                {
                    const int v = cur[px];
                    solid = (size_t)v * 3 + 2 < pal.size() && (pal[v * 3] | pal[v * 3 + 1] | pal[v * 3 + 2]);
                }
                else
                {
                    const int colour = ctype == 4 ? 1 : (ctype == 6 ? 3 : chans);
                    for (int ch = 0; ch < colour; ch++) solid |= sample(ch) != 0;
                }
            }
            mask[(size_t)y * width + x] = solid ? 1 : 0;
        }
        std::swap(prev, cur);
    }
    return true;
}

bool load_uct_image(const UctConfig &uct, Image &img, std::string &err)
{
    std::vector<std::string> files;
    if (!uct.img_files_list.empty() && uct.img_files_list != "Empty")
    {
        std::ifstream f(uct.img_files_list);
        if (!f)
        {
            err = "Could not open file from disc: " + uct.img_files_list;
            return false;
        }
        std::string line;
        while ((int)files.size() < uct.slices && std::getline(f, line)) files.push_back(line);
    }
    else
        for (int s = 0; s < uct.slices; s++)
        {
            std::ostringstream id;
            id << std::setfill('0') << std::setw(uct.digits) << (uct.first_idx + s);
            files.push_back(uct.dir_path + uct.filename + id.str() + uct.extension);
        }
    img = Image();
    for (size_t s = 0; s < files.size(); s++)
    {
        int w = 0, h = 0;
        std::vector<uint8_t> m;
        if (!png_solid_mask(files[s], w, h, m, err)) return false;
        if (s == 0)
        {
            img.nx = w;
            img.ny = h;
            img.labels.reserve((size_t)w * h * files.size());
        }
        else if (w != img.nx || h != img.ny)
        {
            err = files[s] + ": slice size differs from the first slice";
            return false;
        }
        img.labels.insert(img.labels.end(), m.begin(), m.end());
    }
    img.nz = (int)files.size();
    img.n_phases = 1;
    img.source = files.empty() ? "" : files[0];
    if (img.nz == 0)
    {
        err = "uct config names no image slices";
        return false;
    }
    return true;
}

} // namespace rwnmr_host

extern "C" int64_t rwnmr_png_solid_mask(const char *path, int32_t *width, int32_t *height, uint8_t *mask, char *err,
                                        int32_t errlen)
{
    int w = 0, h = 0;
    std::vector<uint8_t> m;
    std::string e;
    if (!path || !rwnmr_host::png_solid_mask(path, w, h, m, e))
    {
        if (err && errlen > 0)
        {
            std::strncpy(err, path ? e.c_str() : "NULL path", (size_t)errlen - 1);
            err[errlen - 1] = 0;
        }
        return -1;
    }
    if (width) *width = w;
    if (height) *height = h;
    if (mask) std::memcpy(mask, m.data(), m.size());
    return (int64_t)m.size();
}
