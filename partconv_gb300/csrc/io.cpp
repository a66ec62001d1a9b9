// io.cpp -- pc.config parser and a minimal RIFF/WAVE reader (host only).
//
// pc.config format (src/pc.config:43-44, parsed by PartConvMulti::setup,
// src/partconvMulti.cpp:36-134 of ebattenberg/partconv):
//   FS buffer_size numInputChannels numOutputChannels numPCs numRepeats
//   then numPCs lines: filename mute inputChannel outputChannel scale M
//                      N0 P0 N1 P1 ... N_{M-1} [P_{M-1}]
// The last level's part count may be omitted and is recomputed from the IR
// length (partconvMulti.cpp:109-110).  numRepeats > 1 appends muted copies
// of every PC (partconvMulti.cpp:118-133).  Tokens after the numPCs lines are
// ignored, as fscanf-driven parsing ignores them.
//
// The WAV reader replaces libsndfile's sf_readf_float for readImpulseResponse
// (src/sndtools.cpp:3-47): channel 0 of 8/16/24/32-bit PCM or 32/64-bit
// float, integers scaled to [-1, 1) by 2^(bits-1).
#include "io.h"

#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace pcg {

static bool parse_int(const std::string& t, int& v) {
    if (t.empty()) return false;
    char* end = nullptr;
    errno = 0;
    long x = std::strtol(t.c_str(), &end, 10);
    if (errno || *end != '\0') return false;
    v = (int)x;
    return true;
}

static bool parse_float(const std::string& t, float& v) {
    if (t.empty()) return false;
    char* end = nullptr;
    errno = 0;
    double x = std::strtod(t.c_str(), &end);
    if (errno || *end != '\0') return false;
    v = (float)x;
    return true;
}

int parse_config(const std::string& text, ConfigFile& cfg, std::string& err) {
    std::istringstream ss(text);
    std::vector<std::string> tok;
    std::string w;
    while (ss >> w) tok.push_back(w);
    size_t i = 0;
    auto next_int = [&](int& v) { return i < tok.size() && parse_int(tok[i], v) ? (++i, true) : false; };
    int hdr[6];
    for (int k = 0; k < 6; ++k) {
        if (!next_int(hdr[k])) {
            err = "error reading config header (FS buffer_size nIn nOut numPCs numRepeats)";
            return 1;
        }
    }
    cfg.fs = hdr[0];
    cfg.buffer_size = hdr[1];
    cfg.n_in = hdr[2];
    cfg.n_out = hdr[3];
    const int npc = hdr[4], nrep = hdr[5];
    if (npc < 1 || nrep < 1 || cfg.n_in < 1 || cfg.n_out < 1 || cfg.buffer_size < 1) {
        err = "config header values must be positive";
        return 1;
    }
    cfg.pcs.clear();
    for (int p = 0; p < npc; ++p) {
        ConfigPC pc;
        if (i >= tok.size()) {
            err = "config ends before PC line " + std::to_string(p + 1);
            return 1;
        }
        pc.file = tok[i++];
        int M = 0;
        if (!next_int(pc.mute) || !next_int(pc.in_ch) || !next_int(pc.out_ch) || i >= tok.size() ||
            !parse_float(tok[i++], pc.scale) || !next_int(M) || M < 1) {
            err = "error reading PC line " + std::to_string(p + 1) + " (file mute in out scale M ...)";
            return 1;
        }
        pc.N.assign(M, 0);
        pc.P.assign(M, 0);
        for (int j = 0; j < M; ++j) {
            if (!next_int(pc.N[j])) {
                err = "error reading block size " + std::to_string(j) + " of PC line " + std::to_string(p + 1);
                return 1;
            }
            if (j < M - 1) {
                if (!next_int(pc.P[j])) {
                    err = "error reading part count " + std::to_string(j) + " of PC line " + std::to_string(p + 1);
                    return 1;
                }
            } else {
                int dummy;
                if (next_int(dummy)) pc.P[j] = dummy;   // optional, ignored
                pc.P[j] = 0;
            }
        }
        if (pc.N[0] != cfg.buffer_size) {
            err = "line " + std::to_string(p + 1) + ": first block size must equal buffer_size";
            return 1;
        }
        cfg.pcs.push_back(pc);
    }
    for (int r = 1; r < nrep; ++r)
        for (int p = 0; p < npc; ++p) {
            ConfigPC c = cfg.pcs[p];
            c.mute = 1;
            cfg.pcs.push_back(c);
        }
    return 0;
}

static uint32_t rd32(const unsigned char* p) { return p[0] | (p[1] << 8) | (p[2] << 16) | ((uint32_t)p[3] << 24); }
static uint16_t rd16(const unsigned char* p) { return (uint16_t)(p[0] | (p[1] << 8)); }

int read_wav_channel0(const std::string& path, std::vector<float>& out, int* sample_rate, std::string& err) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        err = "can't open audio file: " + path;
        return 1;
    }
    std::vector<unsigned char> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    if (buf.size() < 12 || std::memcmp(buf.data(), "RIFF", 4) || std::memcmp(buf.data() + 8, "WAVE", 4)) {
        err = "not a RIFF/WAVE file: " + path;
        return 1;
    }
    int fmt = -1, channels = 0, bits = 0, rate = 0, block_align = 0;
    const unsigned char* data = nullptr;
    size_t data_len = 0;
    size_t pos = 12;
    while (pos + 8 <= buf.size()) {
        const unsigned char* ck = buf.data() + pos;
        uint32_t len = rd32(ck + 4);
        size_t body = pos + 8;
        size_t avail = buf.size() - body;
        if (!std::memcmp(ck, "fmt ", 4) && len >= 16 && avail >= 16) {
            fmt = rd16(ck + 8);
            channels = rd16(ck + 10);
            rate = (int)rd32(ck + 12);
            block_align = rd16(ck + 20);
            bits = rd16(ck + 22);
            if (fmt == 0xFFFE && len >= 26 && avail >= 26) fmt = rd16(ck + 8 + 24);   // extensible subformat
        } else if (!std::memcmp(ck, "data", 4)) {
            data = buf.data() + body;
            data_len = std::min<size_t>(len, avail);
        }
        pos = body + len + (len & 1);
    }
    if (fmt < 0 || !data || channels < 1 || bits < 8) {
        err = "WAV file lacks fmt/data chunks: " + path;
        return 1;
    }
    const int bps = bits / 8;
    if (block_align < channels * bps) block_align = channels * bps;
    const size_t frames = data_len / block_align;
    out.assign(frames, 0.0f);
    for (size_t n = 0; n < frames; ++n) {
        const unsigned char* p = data + n * block_align;   // channel 0
        float v;
        if (fmt == 1) {
            if (bps == 1) v = ((int)p[0] - 128) / 128.0f;
            else if (bps == 2) v = (int16_t)rd16(p) / 32768.0f;
            else if (bps == 3) {
                int32_t s = (int32_t)((uint32_t)p[0] << 8 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 24) >> 8;
                v = (float)s / 8388608.0f;
            } else if (bps == 4) v = (float)((double)(int32_t)rd32(p) / 2147483648.0);
            else {
                err = "unsupported PCM width in " + path;
                return 1;
            }
        } else if (fmt == 3) {
            if (bps == 4) {
                uint32_t u = rd32(p);
                std::memcpy(&v, &u, 4);
            } else if (bps == 8) {
                uint64_t u = (uint64_t)rd32(p) | ((uint64_t)rd32(p + 4) << 32);
                double d;
                std::memcpy(&d, &u, 8);
                v = (float)d;
            } else {
                err = "unsupported float width in " + path;
                return 1;
            }
        } else {
            err = "unsupported WAV encoding in " + path;
            return 1;
        }
        out[n] = v;
    }
    if (sample_rate) *sample_rate = rate;
    return 0;
}

}  // namespace pcg
