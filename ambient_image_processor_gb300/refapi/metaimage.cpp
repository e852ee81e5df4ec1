// MetaImage / raw volume IO (metaimage.hpp).
#include "metaimage.hpp"

#include <cctype>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>

namespace tgvdct_io {
namespace {

std::string trim(const std::string& s) {
    const size_t a = s.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return "";
    const size_t b = s.find_last_not_of(" \t\r\n");
    return s.substr(a, b - a + 1);
}

std::string directory_of(const std::string& path) {
    const size_t k = path.find_last_of('/');
    return k == std::string::npos ? std::string() : path.substr(0, k + 1);
}

bool ends_with(const std::string& s, const std::string& tail) {
    return s.size() >= tail.size() && s.compare(s.size() - tail.size(), tail.size(), tail) == 0;
}

bool host_is_little_endian() {
    const uint16_t one = 1;
    unsigned char b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}

template <class T>
void convert(const unsigned char* src, size_t n, bool swap, std::vector<float>& out) {
    out.resize(n);
    for (size_t i = 0; i < n; ++i) {
        unsigned char b[sizeof(T)];
        std::memcpy(b, src + i * sizeof(T), sizeof(T));
        if (swap)
            for (size_t k = 0; k < sizeof(T) / 2; ++k) std::swap(b[k], b[sizeof(T) - 1 - k]);
        T v;
        std::memcpy(&v, b, sizeof(T));
        out[i] = (float)v;
    }
}

size_t element_size(const std::string& type) {
    if (type == "MET_UCHAR" || type == "MET_CHAR") return 1;
    if (type == "MET_USHORT" || type == "MET_SHORT") return 2;
    if (type == "MET_UINT" || type == "MET_INT" || type == "MET_FLOAT") return 4;
    if (type == "MET_DOUBLE") return 8;
    throw std::runtime_error("unsupported MetaImage ElementType " + type);
}

void parse_doubles(const std::string& s, double* out, int n) {
    std::istringstream in(s);
    for (int k = 0; k < n; ++k)
        if (!(in >> out[k])) break;
}

}  // namespace

Volume read_metaimage(const std::string& path) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("cannot open " + path);
    std::map<std::string, std::string> h;
    std::string line;
    // Header lines "Key = Value"; ElementDataFile is the last one.
    while (std::getline(in, line)) {
        const size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        const std::string key = trim(line.substr(0, eq)), val = trim(line.substr(eq + 1));
        h[key] = val;
        if (key == "ElementDataFile") break;
    }
    if (!h.count("DimSize") || !h.count("ElementType") || !h.count("ElementDataFile"))
        throw std::runtime_error(path + ": not a MetaImage header (DimSize, ElementType, "
                                        "ElementDataFile required)");
    const int ndims = h.count("NDims") ? std::stoi(h["NDims"]) : 3;
    if (ndims < 2 || ndims > 3) throw std::runtime_error(path + ": NDims must be 2 or 3");
    auto is_true = [&](const char* key) {
        if (!h.count(key)) return false;
        std::string v = h[key];
        for (auto& c : v) c = (char)std::tolower((unsigned char)c);
        return v == "true" || v == "1";
    };
    if (is_true("CompressedData")) throw std::runtime_error(path + ": compressed MetaImage data");
    Volume v;
    {
        std::istringstream ds(h["DimSize"]);
        uint32_t d[3] = {1, 1, 1};
        for (int k = 0; k < ndims; ++k)
            if (!(ds >> d[k])) throw std::runtime_error(path + ": bad DimSize");
        v.width = d[0];
        v.height = d[1];
        v.depth = d[2];
    }
    if (h.count("ElementSpacing")) parse_doubles(h["ElementSpacing"], v.spacing, ndims);
    if (h.count("Offset")) parse_doubles(h["Offset"], v.origin, ndims);
    if (h.count("Position")) parse_doubles(h["Position"], v.origin, ndims);
    const std::string type = h["ElementType"];
    const size_t es = element_size(type);
    const bool msb = is_true("BinaryDataByteOrderMSB") || is_true("ElementByteOrderMSB");
    const bool swap = es > 1 && (msb == host_is_little_endian());
    const size_t n = v.count();
    std::vector<unsigned char> raw(n * es);
    const std::string data_file = h["ElementDataFile"];
    if (data_file == "LOCAL") {
        in.read((char*)raw.data(), (std::streamsize)raw.size());
        if ((size_t)in.gcount() != raw.size()) throw std::runtime_error(path + ": truncated data");
    } else {
        const std::string dp = data_file[0] == '/' ? data_file : directory_of(path) + data_file;
        std::ifstream din(dp, std::ios::binary);
        if (!din) throw std::runtime_error("cannot open data file " + dp);
        din.read((char*)raw.data(), (std::streamsize)raw.size());
        if ((size_t)din.gcount() != raw.size()) throw std::runtime_error(dp + ": truncated data");
    }
    const unsigned char* s = raw.data();
    if (type == "MET_UCHAR") convert<uint8_t>(s, n, false, v.voxels);
    else if (type == "MET_CHAR") convert<int8_t>(s, n, false, v.voxels);
    else if (type == "MET_USHORT") convert<uint16_t>(s, n, swap, v.voxels);
    else if (type == "MET_SHORT") convert<int16_t>(s, n, swap, v.voxels);
    else if (type == "MET_UINT") convert<uint32_t>(s, n, swap, v.voxels);
    else if (type == "MET_INT") convert<int32_t>(s, n, swap, v.voxels);
    else if (type == "MET_FLOAT") convert<float>(s, n, swap, v.voxels);
    else convert<double>(s, n, swap, v.voxels);
    return v;
}

void write_metaimage(const std::string& path, const Volume& v) {
    const bool separate = ends_with(path, ".mhd");
    std::string data_name = "LOCAL", data_path;
    if (separate) {
        data_path = path.substr(0, path.size() - 4) + ".raw";
        const size_t k = data_path.find_last_of('/');
        data_name = k == std::string::npos ? data_path : data_path.substr(k + 1);
    }
    std::ofstream out(path, std::ios::binary);
    if (!out) throw std::runtime_error("cannot write " + path);
    const bool three = v.depth > 1;
    const int nd = three ? 3 : 2;
    std::ostringstream hdr;
    hdr.precision(17);
    hdr << "ObjectType = Image\nNDims = " << nd << "\nBinaryData = True\n"
        << "BinaryDataByteOrderMSB = " << (host_is_little_endian() ? "False" : "True") << "\n"
        << "CompressedData = False\n";
    hdr << "Offset =";
    for (int k = 0; k < nd; ++k) hdr << " " << v.origin[k];
    hdr << "\nElementSpacing =";
    for (int k = 0; k < nd; ++k) hdr << " " << v.spacing[k];
    hdr << "\nDimSize = " << v.width << " " << v.height;
    if (three) hdr << " " << v.depth;
    hdr << "\nElementType = MET_FLOAT\nElementDataFile = " << data_name << "\n";
    const std::string hs = hdr.str();
    out.write(hs.data(), (std::streamsize)hs.size());
    if (separate) {
        std::ofstream dout(data_path, std::ios::binary);
        if (!dout) throw std::runtime_error("cannot write " + data_path);
        dout.write((const char*)v.voxels.data(), (std::streamsize)(v.voxels.size() * 4));
    } else {
        out.write((const char*)v.voxels.data(), (std::streamsize)(v.voxels.size() * 4));
    }
    if (!out) throw std::runtime_error("write failed: " + path);
}

Volume read_raw(const std::string& path, uint32_t width, uint32_t height, uint32_t depth) {
    Volume v;
    v.width = width;
    v.height = height;
    v.depth = depth;
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("cannot open " + path);
    std::vector<unsigned char> raw(v.count() * 4);
    in.read((char*)raw.data(), (std::streamsize)raw.size());
    if ((size_t)in.gcount() != raw.size()) throw std::runtime_error(path + ": fewer voxels than WxHxD");
    convert<float>(raw.data(), v.count(), !host_is_little_endian(), v.voxels);
    return v;
}

void write_raw(const std::string& path, const Volume& v) {
    std::ofstream out(path, std::ios::binary);
    if (!out) throw std::runtime_error("cannot write " + path);
    std::vector<float> le(v.voxels);
    if (!host_is_little_endian()) {
        std::vector<float> tmp;
        convert<float>((const unsigned char*)v.voxels.data(), v.voxels.size(), true, tmp);
        le.swap(tmp);
    }
    out.write((const char*)le.data(), (std::streamsize)(le.size() * 4));
    if (!out) throw std::runtime_error("write failed: " + path);
}

Volume read_volume(const std::string& path, const std::string& raw_dims) {
    if (raw_dims.empty()) return read_metaimage(path);
    uint32_t d[3] = {1, 1, 1};
    int k = 0;
    std::string tok;
    std::istringstream in(raw_dims);
    while (k < 3 && std::getline(in, tok, 'x')) d[k++] = (uint32_t)std::stoul(tok);
    if (k < 2) throw std::runtime_error("--raw wants WxH or WxHxD, got " + raw_dims);
    return read_raw(path, d[0], d[1], d[2]);
}

void write_volume(const std::string& path, const Volume& v) {
    if (ends_with(path, ".raw")) write_raw(path, v);
    else write_metaimage(path, v);
}

}  // namespace tgvdct_io
