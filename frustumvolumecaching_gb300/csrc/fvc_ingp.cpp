/*
 * fvc_ingp.cpp - reader of instant-ngp snapshots (.ingp): the second model
 * format of the reference's loader (load_ingp_snapshot, src/loader.cu:146-230).
 *
 * An .ingp file is a msgpack document compressed as a deflate stream (gzip or
 * zlib wrapper, or stored without one).  Both decoders are written here from the published formats
 * (RFC 1951 deflate, RFC 1950/1952 wrappers, the msgpack specification), so
 * the library needs no compression library.  The reader extracts what the
 * reference's loader reads: snapshot.mode, snapshot.nerf.aabb_scale,
 * snapshot.aabb.{min,max}, the encoding / network / rgb_network / dir_encoding
 * configuration, snapshot.params_binary (fp16 network parameters) and
 * snapshot.density_grid_binary (fp16, Morton order per cascade).
 */
#include "fvc_ingp.h"

#include <cstring>
#include <fstream>
#include <map>
#include <memory>

namespace fvc_ingp {
namespace {

/* ---------------------------------------------------------------------- */
/* deflate (RFC 1951)                                                     */
/* ---------------------------------------------------------------------- */
struct BitReader {
    const uint8_t *p;
    size_t n, pos = 0;
    uint32_t bitbuf = 0;
    int bitcnt = 0;
    bool overrun = false;
    int bits(int need)
    {
        while (bitcnt < need) {
            uint32_t byte = 0;
            if (pos < n) byte = p[pos++];
            else overrun = true;
            bitbuf |= byte << bitcnt;
            bitcnt += 8;
        }
        const int v = (int)(bitbuf & ((1u << need) - 1u));
        bitbuf >>= need;
        bitcnt -= need;
        return v;
    }
    void align()
    {
        bitbuf = 0;
        bitcnt = 0;
    }
};

/* canonical Huffman code: counts per length and symbols in code order */
struct Huffman {
    uint16_t count[16] = {};
    std::vector<uint16_t> symbol;
    bool build(const uint8_t *lengths, int n)
    {
        for (int i = 0; i < 16; ++i) count[i] = 0;
        for (int i = 0; i < n; ++i) count[lengths[i]]++;
        count[0] = 0;
        int left = 1;
        for (int len = 1; len < 16; ++len) {
            left = 2 * left - count[len];
            if (left < 0) return false; /* over-subscribed */
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int len = 1; len < 15; ++len) offs[len + 1] = offs[len] + count[len];
        symbol.assign(n, 0);
        for (int i = 0; i < n; ++i)
            if (lengths[i]) symbol[offs[lengths[i]]++] = (uint16_t)i;
        return true;
    }
    /* one symbol, reading the code bit by bit (codes are stored MSB first) */
    int decode(BitReader &br) const
    {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; ++len) {
            code |= br.bits(1);
            const int c = count[len];
            if (code - c < first) return symbol[index + (code - first)];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
            if (br.overrun) return -1;
        }
        return -1;
    }
};

constexpr uint16_t LEN_BASE[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
constexpr uint8_t LEN_EXTRA[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
constexpr uint16_t DIST_BASE[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769,
                                    1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
constexpr uint8_t DIST_EXTRA[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_codes(BitReader &br, const Huffman &lit, const Huffman &dist, std::vector<uint8_t> &out, std::string &err)
{
    for (;;) {
        int sym = lit.decode(br);
        if (sym < 0) { err = "deflate: bad literal/length code"; return false; }
        if (sym < 256) { out.push_back((uint8_t)sym); continue; }
        if (sym == 256) return true;
        sym -= 257;
        if (sym >= 29) { err = "deflate: bad length symbol"; return false; }
        const int len = LEN_BASE[sym] + br.bits(LEN_EXTRA[sym]);
        const int ds = dist.decode(br);
        if (ds < 0 || ds >= 30) { err = "deflate: bad distance code"; return false; }
        const size_t d = (size_t)DIST_BASE[ds] + (size_t)br.bits(DIST_EXTRA[ds]);
        if (d > out.size()) { err = "deflate: distance beyond the output"; return false; }
        const size_t from = out.size() - d;
        for (int i = 0; i < len; ++i) out.push_back(out[from + i]);
        if (br.overrun) { err = "deflate: truncated stream"; return false; }
    }
}

bool inflate_raw(const uint8_t *in, size_t n, std::vector<uint8_t> &out, size_t &consumed, std::string &err)
{
    BitReader br{in, n};
    for (int last = 0; !last;) {
        last = br.bits(1);
        const int type = br.bits(2);
        if (type == 0) { /* stored */
            br.align();
            if (br.pos + 4 > n) { err = "deflate: truncated stored block"; return false; }
            const unsigned len = in[br.pos] | (in[br.pos + 1] << 8), nlen = in[br.pos + 2] | (in[br.pos + 3] << 8);
            br.pos += 4;
            if ((len ^ 0xFFFFu) != nlen || br.pos + len > n) { err = "deflate: bad stored block"; return false; }
            out.insert(out.end(), in + br.pos, in + br.pos + len);
            br.pos += len;
        } else if (type == 1) { /* fixed codes */
            uint8_t l[288], d[30];
            for (int i = 0; i < 144; ++i) l[i] = 8;
            for (int i = 144; i < 256; ++i) l[i] = 9;
            for (int i = 256; i < 280; ++i) l[i] = 7;
            for (int i = 280; i < 288; ++i) l[i] = 8;
            for (int i = 0; i < 30; ++i) d[i] = 5;
            Huffman lit, dist;
            lit.build(l, 288);
            dist.build(d, 30);
            if (!inflate_codes(br, lit, dist, out, err)) return false;
        } else if (type == 2) { /* dynamic codes */
            const int nlen = br.bits(5) + 257, ndist = br.bits(5) + 1, ncode = br.bits(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {};
            for (int i = 0; i < ncode; ++i) cl[order[i]] = (uint8_t)br.bits(3);
            Huffman clh;
            if (!clh.build(cl, 19)) { err = "deflate: bad code-length code"; return false; }
            uint8_t lengths[320] = {};
            for (int i = 0; i < nlen + ndist;) {
                const int sym = clh.decode(br);
                if (sym < 0) { err = "deflate: bad code length"; return false; }
                if (sym < 16) { lengths[i++] = (uint8_t)sym; continue; }
                int rep = 0;
                uint8_t val = 0;
                if (sym == 16) {
                    if (i == 0) { err = "deflate: repeat without a length"; return false; }
                    val = lengths[i - 1];
                    rep = 3 + br.bits(2);
                } else if (sym == 17) {
                    rep = 3 + br.bits(3);
                } else {
                    rep = 11 + br.bits(7);
                }
                if (i + rep > nlen + ndist) { err = "deflate: too many code lengths"; return false; }
                while (rep--) lengths[i++] = val;
            }
            Huffman lit, dist;
            if (!lit.build(lengths, nlen) || !dist.build(lengths + nlen, ndist)) { err = "deflate: bad code lengths"; return false; }
            if (!inflate_codes(br, lit, dist, out, err)) return false;
        } else {
            err = "deflate: reserved block type";
            return false;
        }
        if (br.overrun) { err = "deflate: truncated stream"; return false; }
    }
    consumed = br.pos;
    return true;
}

/* gzip (RFC 1952) or zlib (RFC 1950) wrapper around one deflate stream */
bool decompress(const std::vector<uint8_t> &in, std::vector<uint8_t> &out, std::string &err)
{
    size_t start = 0;
    if (in.size() >= 10 && in[0] == 0x1f && in[1] == 0x8b) {
        if (in[2] != 8) { err = "gzip: not deflate"; return false; }
        const uint8_t flg = in[3];
        start = 10;
        if (flg & 4) { /* FEXTRA */
            if (start + 2 > in.size()) { err = "gzip: truncated header"; return false; }
            start += 2 + (in[start] | (in[start + 1] << 8));
        }
        if (flg & 8) while (start < in.size() && in[start++]) {} /* FNAME */
        if (flg & 16) while (start < in.size() && in[start++]) {} /* FCOMMENT */
        if (flg & 2) start += 2; /* FHCRC */
    } else if (in.size() >= 2 && (in[0] & 0x0f) == 8 && (in[0] >> 4) <= 7 && ((in[0] << 8) | in[1]) % 31 == 0) {
        if (in[1] & 0x20) { err = "zlib: preset dictionary not supported"; return false; }
        start = 2;
    } else { /* no wrapper: an uncompressed msgpack document, as the reference's stream reader passes it */
        out = in;
        return true;
    }
    if (start >= in.size()) { err = "truncated stream header"; return false; }
    size_t consumed = 0;
    out.clear();
    out.reserve(in.size() * 2);
    return inflate_raw(in.data() + start, in.size() - start, out, consumed, err);
}

/* ---------------------------------------------------------------------- */
/* msgpack                                                                */
/* ---------------------------------------------------------------------- */
struct MVal {
    enum Kind { NIL, BOOL, INT, FLOAT, STR, BIN, ARR, MAP } kind = NIL;
    bool b = false;
    long long i = 0;
    double f = 0.0;
    std::string s;                 /* STR text or BIN bytes */
    std::vector<MVal> arr;
    std::map<std::string, MVal> map;
    const MVal *get(const std::string &k) const
    {
        if (kind != MAP) return nullptr;
        auto it = map.find(k);
        return it == map.end() ? nullptr : &it->second;
    }
    double num(double dflt) const { return kind == INT ? (double)i : kind == FLOAT ? f : dflt; }
};

struct MParser {
    const uint8_t *p, *e;
    bool ok = true;
    int depth = 0;
    uint64_t be(int nb)
    {
        if (e - p < nb) { ok = false; return 0; }
        uint64_t v = 0;
        for (int k = 0; k < nb; ++k) v = (v << 8) | *p++;
        return v;
    }
    void raw(std::string &dst, uint64_t n)
    {
        if ((uint64_t)(e - p) < n) { ok = false; return; }
        dst.assign(reinterpret_cast<const char *>(p), (size_t)n);
        p += n;
    }
    MVal parse()
    {
        MVal v;
        if (!ok || p >= e || ++depth > 64) { ok = false; return v; }
        const uint8_t c = *p++;
        auto arr = [&](uint64_t n) {
            v.kind = MVal::ARR;
            for (uint64_t k = 0; k < n && ok; ++k) v.arr.push_back(parse());
        };
        auto map = [&](uint64_t n) {
            v.kind = MVal::MAP;
            for (uint64_t k = 0; k < n && ok; ++k) {
                MVal key = parse();
                MVal val = parse();
                if (key.kind == MVal::STR) v.map[key.s] = std::move(val);
            }
        };
        if (c <= 0x7f) { v.kind = MVal::INT; v.i = c; }
        else if (c >= 0xe0) { v.kind = MVal::INT; v.i = (int8_t)c; }
        else if ((c & 0xf0) == 0x80) map(c & 0x0f);
        else if ((c & 0xf0) == 0x90) arr(c & 0x0f);
        else if ((c & 0xe0) == 0xa0) { v.kind = MVal::STR; raw(v.s, c & 0x1f); }
        else switch (c) {
            case 0xc0: break;
            case 0xc2: v.kind = MVal::BOOL; v.b = false; break;
            case 0xc3: v.kind = MVal::BOOL; v.b = true; break;
            case 0xc4: v.kind = MVal::BIN; raw(v.s, be(1)); break;
            case 0xc5: v.kind = MVal::BIN; raw(v.s, be(2)); break;
            case 0xc6: v.kind = MVal::BIN; raw(v.s, be(4)); break;
            case 0xc7: { const uint64_t n = be(1); be(1); std::string t; raw(t, n); break; } /* ext: skipped */
            case 0xc8: { const uint64_t n = be(2); be(1); std::string t; raw(t, n); break; }
            case 0xc9: { const uint64_t n = be(4); be(1); std::string t; raw(t, n); break; }
            case 0xca: { v.kind = MVal::FLOAT; const uint32_t u = (uint32_t)be(4); float f; std::memcpy(&f, &u, 4); v.f = f; break; }
            case 0xcb: { v.kind = MVal::FLOAT; const uint64_t u = be(8); std::memcpy(&v.f, &u, 8); break; }
            case 0xcc: v.kind = MVal::INT; v.i = (long long)be(1); break;
            case 0xcd: v.kind = MVal::INT; v.i = (long long)be(2); break;
            case 0xce: v.kind = MVal::INT; v.i = (long long)be(4); break;
            case 0xcf: v.kind = MVal::INT; v.i = (long long)be(8); break;
            case 0xd0: v.kind = MVal::INT; v.i = (int8_t)be(1); break;
            case 0xd1: v.kind = MVal::INT; v.i = (int16_t)be(2); break;
            case 0xd2: v.kind = MVal::INT; v.i = (int32_t)be(4); break;
            case 0xd3: v.kind = MVal::INT; v.i = (long long)be(8); break;
            case 0xd4: be(1); be(1); break; /* fixext: skipped */
            case 0xd5: be(1); be(2); break;
            case 0xd6: be(1); be(4); break;
            case 0xd7: be(1); be(8); break;
            case 0xd8: { be(1); std::string t; raw(t, 16); break; }
            case 0xd9: v.kind = MVal::STR; raw(v.s, be(1)); break;
            case 0xda: v.kind = MVal::STR; raw(v.s, be(2)); break;
            case 0xdb: v.kind = MVal::STR; raw(v.s, be(4)); break;
            case 0xdc: arr(be(2)); break;
            case 0xdd: arr(be(4)); break;
            case 0xde: map(be(2)); break;
            case 0xdf: map(be(4)); break;
            default: ok = false; break;
        }
        --depth;
        return v;
    }
};

int int_or(const MVal *m, const char *key, int dflt)
{
    const MVal *v = m ? m->get(key) : nullptr;
    return v ? (int)v->num(dflt) : dflt;
}

const MVal *path(const MVal &root, std::initializer_list<const char *> keys)
{
    const MVal *v = &root;
    for (const char *k : keys) {
        v = v->get(k);
        if (!v) return nullptr;
    }
    return v;
}

}  // namespace

bool read_snapshot(const std::string &file, Snapshot &out, std::string &err)
{
    std::ifstream f(file, std::ios::binary);
    if (!f) { err = "Could not load snapshot file!"; return false; }
    std::vector<uint8_t> packed((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    std::vector<uint8_t> doc;
    if (!decompress(packed, doc, err)) { err = file + ": " + err; return false; }
    MParser mp{doc.data(), doc.data() + doc.size()};
    const MVal root = mp.parse();
    if (!mp.ok || root.kind != MVal::MAP) { err = file + ": not a msgpack map"; return false; }
    const MVal *snap = root.get("snapshot");
    if (!snap) { err = "File '" + file + "' does not contain a snapshot."; return false; }
    const MVal *mode = snap->get("mode");
    if (!mode || mode->kind != MVal::STR || mode->s != "nerf") { err = "File '" + file + "' does not contain a nerf snapshot."; return false; }
    const MVal *scale = path(*snap, {"nerf", "aabb_scale"});
    const MVal *amin = path(*snap, {"aabb", "min"}), *amax = path(*snap, {"aabb", "max"});
    const MVal *params = snap->get("params_binary"), *grid = snap->get("density_grid_binary");
    if (!scale || !amin || !amax || !params || !grid || amin->arr.size() != 3 || amax->arr.size() != 3 ||
        params->kind != MVal::BIN || grid->kind != MVal::BIN) {
        err = file + ": snapshot lacks nerf.aabb_scale, aabb, params_binary or density_grid_binary";
        return false;
    }
    out.aabb_scale = (int)scale->num(1);
    for (int k = 0; k < 3; ++k) {
        out.aabb_min[k] = (float)amin->arr[k].num(0);
        out.aabb_max[k] = (float)amax->arr[k].num(0);
    }
    const MVal *enc = root.get("encoding"), *net = root.get("network"), *rgb = root.get("rgb_network");
    if (!enc || !net || !rgb) { err = file + ": missing encoding / network / rgb_network"; return false; }
    out.n_levels = int_or(enc, "n_levels", 16);
    out.n_features = int_or(enc, "n_features_per_level", 2);
    out.log2_hashmap_size = int_or(enc, "log2_hashmap_size", 19);
    out.base_resolution = int_or(enc, "base_resolution", 16);
    out.base_neurons = int_or(net, "n_neurons", 64);
    out.base_hidden = int_or(net, "n_hidden_layers", 1);
    out.head_neurons = int_or(rgb, "n_neurons", 64);
    out.head_hidden = int_or(rgb, "n_hidden_layers", 2);
    out.sh_degree = 4;
    if (const MVal *nested = path(root, {"dir_encoding", "nested"}))
        if (nested->kind == MVal::ARR && !nested->arr.empty()) out.sh_degree = int_or(&nested->arr[0], "degree", 4);
    if (params->s.size() % 2 || grid->s.size() % 2) { err = file + ": odd fp16 blob size"; return false; }
    out.params.resize(params->s.size() / 2);
    std::memcpy(out.params.data(), params->s.data(), params->s.size());
    out.density_grid.resize(grid->s.size() / 2);
    std::memcpy(out.density_grid.data(), grid->s.data(), grid->s.size());
    return true;
}

}  // namespace fvc_ingp
