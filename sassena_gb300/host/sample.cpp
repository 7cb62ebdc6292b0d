#include "sample.hpp"

#include <algorithm>
#include <cstring>
#include <fstream>
#include <regex>
#include <sstream>
#include <stdexcept>

namespace sassgpu {

namespace {

int32_t read_i32(std::ifstream& f) {
    int32_t v = 0;
    f.read(reinterpret_cast<char*>(&v), 4);
    if (!f) throw std::runtime_error("truncated DCD file");
    return v;
}

}  // namespace

bool DcdFile::detect(const std::string& path) {
    // DCDFrameset::detect (frames.cpp:359-370): int 84 at bytes 0 and 88, "CORD" at 4.
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    unsigned char buf[92];
    f.read(reinterpret_cast<char*>(buf), 92);
    if (!f) return false;
    const unsigned char fp1[4] = {0x54, 0, 0, 0}, fp2[4] = {0x43, 0x4f, 0x52, 0x44};
    return memcmp(buf, fp1, 4) == 0 && memcmp(buf + 88, fp1, 4) == 0 && memcmp(buf + 4, fp2, 4) == 0;
}

void DcdFile::open(const std::string& p) {
    path = p;
    if (!detect(p)) throw std::runtime_error("file '" + p + "' appears to not be a DCD file. INT Magic failed");
    std::ifstream f(p, std::ios::binary);
    // header record (DCDHeader, frames.hpp:152-164): 84 | "CORD" | NSET ISTART NSAVC
    // 6*int float(DELTA) ext1 ext2 ... | 84, i.e. ints 2 (frames), 12 and 13 (blocks)
    int32_t hdr[14];
    f.read(reinterpret_cast<char*>(hdr), sizeof(hdr));
    nframes_header = (size_t)hdr[2];
    ext_block1 = hdr[12] != 0;
    ext_block2 = hdr[13] != 0;
    f.seekg(23 * 4, std::ios::beg);  // title record
    int32_t m = read_i32(f);
    f.seekg(m, std::ios::cur);
    read_i32(f);
    read_i32(f);
    int32_t noa = read_i32(f);
    read_i32(f);
    if (noa <= 0) throw std::runtime_error("DCD file '" + p + "' has no atoms");
    natoms = (size_t)noa;
    first_frame_pos = (uint64_t)f.tellg();
    uint64_t pos = 0;
    if (ext_block1) pos += 4 + 48 + 4;
    x_off = pos + 4;
    pos += 4 + 4 * natoms + 4;
    y_off = pos + 4;
    pos += 4 + 4 * natoms + 4;
    z_off = pos + 4;
    pos += 4 + 4 * natoms + 4;
    if (ext_block2) pos += 4 + 4 * natoms + 4;
    frame_bytes = pos;
    // the header's frame count, checked against the file size
    f.seekg(0, std::ios::end);
    uint64_t size = (uint64_t)f.tellg();
    if (first_frame_pos + nframes_header * frame_bytes > size)
        throw std::runtime_error("DCD file '" + p + "' is truncated: header announces " +
                                 std::to_string(nframes_header) + " frames");
    frame_pos.clear();
    for (size_t i = 0; i < nframes_header; ++i) frame_pos.push_back(first_frame_pos + i * frame_bytes);
}

void DcdFile::select(size_t first, size_t last, bool last_set, size_t stride) {
    // FileFrameset::trim_index (frames.cpp:232-255): note the stride applies to the
    // absolute frame index, not the index relative to `first`.
    std::vector<uint64_t> keep;
    for (size_t i = 0; i < frame_pos.size(); ++i) {
        if (i < first) continue;
        if (last_set && i > last) break;
        if (i % stride == 0) keep.push_back(frame_pos[i]);
    }
    frame_pos.swap(keep);
}

void DcdFile::read_frame(size_t i, float* x, float* y, float* z) const {
    std::ifstream f(path, std::ios::binary);
    const uint64_t base = frame_pos.at(i);
    float* dst[3] = {x, y, z};
    uint64_t off[3] = {x_off, y_off, z_off};
    for (int k = 0; k < 3; ++k) {
        f.seekg((std::streamoff)(base + off[k]), std::ios::beg);
        f.read(reinterpret_cast<char*>(dst[k]), (std::streamsize)(4 * natoms));
        if (!f) throw std::runtime_error("truncated DCD frame in " + path);
    }
}

std::map<std::string, std::vector<size_t>> read_ndx_groups(const std::string& path, const std::string& selector,
                                                          const std::string& expression) {
    // AtomselectionReader::read_ndx, atomselection_reader.cpp:33-80: "[ name ]" opens a group
    // (the name is the first token after "[", the closing bracket included when no space
    // separates it); following lines hold 1-based indices, kept for groups whose name matches
    if (selector != "name") throw std::runtime_error("NDX Atomselection only supports selection by 'name' at the moment");
    std::ifstream in(path);
    if (!in) throw std::runtime_error("Couldn't open selection file: " + path);
    std::regex expr(expression);
    std::map<std::string, std::vector<size_t>> groups;
    std::string line, name;
    while (std::getline(in, line)) {
        const size_t pos = line.find('[');
        if (pos != std::string::npos) {
            const size_t pos2 = line.find(']');
            if (pos2 == std::string::npos) throw std::runtime_error("ndx file is missing closing bracket");
            std::istringstream cs(line.substr(pos + 1, pos2 - pos));
            std::string token;
            cs >> token;
            name = trim(token);
        } else if (!name.empty() && std::regex_match(name, expr)) {
            std::istringstream ls(line);
            long long v;
            while (ls >> v) {
                if (v < 1) break;  // the reference reads size_t: zero or negatives stop the line
                groups[name].push_back((size_t)v - 1);
            }
        }
    }
    return groups;
}

std::vector<size_t> read_pdb_selection(const std::string& path, const std::string& selector,
                                       const std::string& expression) {
    // AtomselectionReader::read_pdb, atomselection_reader.cpp:82-120: ATOM records whose beta
    // (columns 61-66) or segid (73-76) field, trimmed, matches the expression
    if (selector != "beta" && selector != "segid")
        throw std::runtime_error("PDB Atomselection only supports beta and segid at the moment");
    std::ifstream in(path);
    if (!in) throw std::runtime_error("Couldn't open selection file: " + path);
    std::regex expr(expression);
    std::vector<size_t> ids;
    std::string line;
    size_t n = 0;
    while (std::getline(in, line)) {
        if (line.compare(0, 6, "ATOM  ") != 0) continue;
        const size_t pos = selector == "beta" ? 60 : 72, len = selector == "beta" ? 6 : 4;
        const std::string v = trim(line.size() > pos ? line.substr(pos, len) : std::string());
        if (std::regex_match(v, expr)) ids.push_back(n);
        ++n;
    }
    return ids;
}

void write_dcd(const std::string& path, const float* frames, size_t nf, size_t na) {
    std::ofstream out(path, std::ios::binary | std::ios::trunc);
    if (!out) throw std::runtime_error("Couldn't open dump file: " + path);
    auto i32 = [&](int32_t v) { out.write(reinterpret_cast<const char*>(&v), 4); };
    // header record: "CORD", frames, start 0, interval 1, 6 zeros, timestep 1.0f, unit-cell
    // block on, fourth-dimension block off, 7 zeros, CHARMM version 24
    i32(84);
    out.write("CORD", 4);
    i32((int32_t)nf);
    i32(0);
    i32(1);
    for (int k = 0; k < 6; ++k) i32(0);
    const float dt = 1.0f;
    out.write(reinterpret_cast<const char*>(&dt), 4);
    i32(1);
    i32(0);
    for (int k = 0; k < 7; ++k) i32(0);
    i32(24);
    i32(84);
    i32(4);  // title record with no title lines
    i32(0);
    i32(4);
    i32(4);  // atom count record
    i32((int32_t)na);
    i32(4);
    std::vector<float> col(na);
    const double cell[6] = {0, 0, 0, 0, 0, 0};
    for (size_t f = 0; f < nf; ++f) {
        i32(48);
        out.write(reinterpret_cast<const char*>(cell), 48);
        i32(48);
        for (int k = 0; k < 3; ++k) {
            for (size_t j = 0; j < na; ++j) col[j] = frames[(f * na + j) * 3 + k];
            i32((int32_t)(4 * na));
            out.write(reinterpret_cast<const char*>(col.data()), (std::streamsize)(4 * na));
            i32((int32_t)(4 * na));
        }
    }
    if (!out) throw std::runtime_error("write error on dump file: " + path);
}

void Sample::init(const Params& p, Database& db) {
    if (p.structure_format != "pdb") throw std::runtime_error("structure format not supported: " + p.structure_format);
    std::ifstream in(p.structure_filepath);
    if (!in) throw std::runtime_error("Couldn't open structure file: " + p.structure_filepath);
    std::string line;
    std::map<std::string, size_t> cache;
    while (std::getline(in, line)) {
        if (line.compare(0, 6, "ATOM  ") != 0) continue;
        std::string pdbname = trim(line.size() > 12 ? line.substr(12, 4) : std::string());
        auto it = cache.find(pdbname);
        if (it == cache.end()) it = cache.emplace(pdbname, db.id(db.label_for_pdb_name(pdbname))).first;
        atom_ids.push_back(it->second);
    }
    if (atom_ids.empty()) throw std::runtime_error("no ATOM records in " + p.structure_filepath);
    const size_t na = atom_ids.size();
    for (const SelectionParams& s : p.selections) {
        std::vector<size_t> idx;
        if (s.type == "index") {
            idx = s.ids;
        } else if (s.type == "range") {
            if (s.to < s.from) throw std::runtime_error("Range Atomselection specified is negative range!");
            for (size_t i = s.from; i <= s.to; ++i) idx.push_back(i);
        } else if (s.type == "lexical") {
            // atoms whose database label matches the expression (atoms.cpp:129-144 selects by
            // label; this build returns atom indices)
            std::regex e(s.expression);
            for (size_t i = 0; i < na; ++i)
                if (std::regex_match(db.labels[atom_ids[i]], e)) idx.push_back(i);
        } else if (s.type == "file") {
            if (s.format == "ndx") {  // every matching group becomes a selection of its own name
                for (auto& g : read_ndx_groups(s.filepath, s.selector, s.expression)) {
                    for (size_t i : g.second)
                        if (i >= na) throw std::runtime_error("ndx group " + g.first + " refers to atom " + std::to_string(i));
                    selections[g.first == "system" ? "system_RENAMED_BY_SASSENA" : g.first] = g.second;
                }
                continue;
            } else if (s.format == "pdb") {
                idx = read_pdb_selection(s.filepath, s.selector, s.expression);
            } else {
                throw std::runtime_error("Selection file format not understood");
            }
        }
        for (size_t i : idx)
            if (i >= na) throw std::runtime_error("selection " + s.name + " refers to atom " + std::to_string(i));
        std::string name = s.name == "system" ? "system_RENAMED_BY_SASSENA" : s.name;
        selections[name] = idx;
    }
    std::vector<size_t> all(na);
    for (size_t i = 0; i < na; ++i) all[i] = i;
    selections["system"] = all;

    auto add_dcd = [&](const std::string& path, const FramesetParams& fs, size_t clones) {
        DcdFile d;
        d.open(path);
        if (d.natoms != na)  // coordinate_sets.cpp:250-255
            throw std::runtime_error("Atom number mismatch (dcd) " + std::to_string(d.natoms) + " vs. (pdb) " +
                                     std::to_string(na));
        d.select(fs.first, fs.last, fs.last_set, fs.stride);
        for (size_t c = 0; c < clones; ++c) {
            framesets.push_back(d);
            nframes += d.frame_pos.size();
        }
    };
    for (const FramesetParams& fs : p.framesets) {
        if (fs.clones == 0) continue;
        if (fs.format == "dcd") {
            add_dcd(fs.filepath, fs, fs.clones);
        } else if (fs.format == "dcdlist") {
            // Frames::add_frameset "dcdlist" (frames.cpp:71-85): whitespace-separated DCD paths,
            // taken as written; tokens starting with '#' are skipped; each file `clones` times
            std::ifstream list(fs.filepath);
            if (!list) throw std::runtime_error("Couldn't open frameset list: " + fs.filepath);
            std::string tok;
            while (list >> tok) {
                if (!tok.empty() && tok[0] == '#') continue;
                for (size_t c = 0; c < fs.clones; ++c) add_dcd(tok, fs, 1);
            }
        } else {
            throw std::runtime_error("frameset format not supported by this build: " + fs.format);
        }
    }
    if (nframes == 0) throw std::runtime_error("Number of frames must not be negative or zero!");
}

const std::vector<size_t>& Sample::selection(const std::string& name) const {
    auto it = selections.find(name);
    if (it == selections.end()) throw std::runtime_error("unknown selection: " + name);
    return it->second;
}

std::vector<float> Sample::stage(const std::string& target) const {
    std::vector<float> out(nframes * selection(target).size() * 3);
    stage_into(target, out.data());
    return out;
}

void Sample::stage_into(const std::string& target, float* out) const {
    const std::vector<size_t>& sel = selection(target);
    const size_t na_all = atom_ids.size(), na = sel.size();
    std::vector<float> x(na_all), y(na_all), z(na_all);
    size_t f = 0;
    for (const DcdFile& d : framesets)
        for (size_t i = 0; i < d.frame_pos.size(); ++i, ++f) {
            d.read_frame(i, x.data(), y.data(), z.data());
            float* o = out + f * na * 3;
            for (size_t n = 0; n < na; ++n) {
                o[3 * n] = x[sel[n]];
                o[3 * n + 1] = y[sel[n]];
                o[3 * n + 2] = z[sel[n]];
            }
        }
}

}  // namespace sassgpu
