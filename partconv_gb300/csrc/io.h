// io.h -- pc.config parsing and WAV reading (host only).
#pragma once
#include <string>
#include <vector>

namespace pcg {

struct ConfigPC {
    std::string file;
    int mute = 0, in_ch = 0, out_ch = 0;
    float scale = 1.0f;
    std::vector<int> N, P;
};

struct ConfigFile {
    int fs = 0, buffer_size = 0, n_in = 0, n_out = 0;
    std::vector<ConfigPC> pcs;   // repeats appended, muted
};

int parse_config(const std::string& text, ConfigFile& cfg, std::string& err);
int read_wav_channel0(const std::string& path, std::vector<float>& out, int* sample_rate, std::string& err);

}  // namespace pcg
