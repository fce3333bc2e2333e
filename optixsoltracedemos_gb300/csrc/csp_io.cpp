// csp_io.cpp -- SolTrace .stinput reader and the hit-record CSV writer (host only).
//
// Reader: the reference's SolTraceSystem::read_st_input and helpers (lib/soltrace_system.cpp:
// 186-206, 495-846), same accepted grammar and the same element mapping:
//   * file must start with '#'; SUN line gives the sun angle as SIGMA * 0.001 whatever the shape
//     letter (pillbox half angle), the XYZ line the sun vector, USER SHAPE DATA lines are skipped;
//   * OPTICS LIST: each "OPTICAL PAIR" is followed by two OPTICAL surface lines (reflectivity /
//     transmissivity tables skipped); the reference discards the values, and so does this reader
//     unless CSP_STINPUT_APPLY_OPTICS asks to apply the front surface's reflectivity and RMS slope /
//     specularity errors (mrad) to the elements that name the pair;
//   * STAGE LIST: each stage line gives its element count, then a name line, then the elements;
//   * element lines (>= 29 tab-separated tokens): 'c' aperture with 'f' surface = cylinder cap,
//     skipped; 'l' aperture with 't' surface = cylinder (radius 1/tok[18], length tok[11], origin y
//     shifted by the radius); 'r' aperture = rectangle tok[9] x tok[10]; 'p' surface = parabolic
//     (tok[18], tok[19]); 'f' = flat; anything else is an error.
// Writer: SolTraceSystem::write_output (lib/soltrace_system.cpp:208-264): header
//   "number,stage,loc_x,loc_y,loc_z", one row per record, a record whose x, y, z are all zero is
//   a marker that ends the current ray, rays are numbered from 1 in order, values printed as the
//   C++ stream prints floats (6 significant digits, %g style; format_g6, csp_format.h).  Blocks of
//   rays are formatted in parallel threads starting from the writer state of their first ray, then
//   written in order; the start states of the next batch of blocks and the writing of the last one
//   overlap the formatting of the current one.
//   CSP_OUT_STAGED leaves out the rows of rays that reach the receiver straight from the sun, as
//   scripts/post_processing/clean_direct_sun.py does to the written file.
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "csp_c_api.h"
#include "csp_format.h"
#include "csp_system.h"

namespace csp {
namespace {

struct LineReader {
    FILE* fp;
    bool eof = false;
    std::string line;
    explicit LineReader(FILE* f) : fp(f) {}
    // fgets of up to 1023 chars with a trailing "\n" / "\r\n" removed (read_line)
    const char* next() {
        char buf[1024];
        if (!std::fgets(buf, sizeof buf, fp)) {
            eof = true;
            line.clear();
            return line.c_str();
        }
        size_t n = std::strlen(buf);
        if (n > 0 && buf[n - 1] == '\n') buf[--n] = 0;
        if (n > 0 && buf[n - 1] == '\r') buf[--n] = 0;
        line.assign(buf, n);
        return line.c_str();
    }
};

// split on tabs keeping empty tokens; no token after a trailing delimiter (split(..., true, false))
std::vector<std::string> split_tabs(const std::string& s) {
    std::vector<std::string> out;
    size_t pos = 0;
    while (pos < s.size()) {
        size_t t = s.find('\t', pos);
        if (t == std::string::npos) {
            out.push_back(s.substr(pos));
            break;
        }
        out.push_back(s.substr(pos, t - pos));
        pos = t + 1;
    }
    return out;
}

struct OpticSurface {
    double reflectivity = 1.0, slope_mrad = 0.0, spec_mrad = 0.0;
};

struct Parsed {
    std::vector<csp_element> elements;
    std::vector<std::string> optic_of;  // optic name per element
    std::map<std::string, OpticSurface> optics;
    double sun[3] = {0, 0, 1};
    double sun_angle = 0.0;
};

bool read_optic_surface(LineReader& r, OpticSurface* out, std::string& err) {
    auto parts = split_tabs(r.next());
    if (parts.size() < 15) {
        err = "too few tokens for optical surface: " + std::to_string(parts.size());
        return false;
    }
    out->reflectivity = std::atof(parts[5].c_str());
    out->slope_mrad = std::atof(parts[7].c_str());
    out->spec_mrad = std::atof(parts[8].c_str());
    int refl_n = 0, trans_n = 0;
    bool use_refl = false, use_trans = false;
    if (parts.size() >= 17) {
        use_refl = std::atoi(parts[15].c_str()) > 0;
        refl_n = std::atoi(parts[16].c_str());
        if (parts.size() >= 19) {
            use_trans = std::atoi(parts[17].c_str()) > 0;
            trans_n = std::atoi(parts[18].c_str());
        }
    }
    if (use_refl)
        for (int i = 0; i < refl_n; ++i) r.next();
    if (use_trans)
        for (int i = 0; i < trans_n; ++i) r.next();
    return true;
}

bool read_element(LineReader& r, Parsed& P, std::string& err) {
    auto tok = split_tabs(r.next());
    if (tok.size() < 29) {
        err = "too few tokens for element: " + std::to_string(tok.size());
        return false;
    }
    const char ap = tok[8].empty() ? 0 : tok[8][0];
    const char sf = tok[17].empty() ? 0 : tok[17][0];
    if (ap == 'c' && sf == 'f') return true;  // cylinder end cap: skipped
    csp_element e;
    std::memset(&e, 0, sizeof e);
    e.origin[0] = std::atof(tok[1].c_str());
    e.origin[1] = std::atof(tok[2].c_str());
    e.origin[2] = std::atof(tok[3].c_str());
    const bool cyl = (ap == 'l' && sf == 't');
    if (cyl) e.origin[1] += 1 / std::atof(tok[18].c_str());
    e.aim_point[0] = std::atof(tok[4].c_str());
    e.aim_point[1] = std::atof(tok[5].c_str());
    e.aim_point[2] = std::atof(tok[6].c_str());
    e.zrot_deg = std::atof(tok[7].c_str());
    e.aperture = CSP_APERTURE_RECTANGLE;
    if (ap == 'r') {
        e.width = std::atof(tok[9].c_str());
        e.height = std::atof(tok[10].c_str());
    } else if (cyl) {
        e.width = 2 * (1 / std::atof(tok[18].c_str()));
        e.height = std::atof(tok[11].c_str());
    } else {
        err = "aperture type not implemented: " + tok[8];
        return false;
    }
    if (sf == 'p') {
        e.surface = CSP_SURFACE_PARABOLIC;
        e.curv_x = std::atof(tok[18].c_str());
        e.curv_y = std::atof(tok[19].c_str());
    } else if (cyl) {
        e.surface = CSP_SURFACE_CYLINDER;
    } else if (sf == 'f') {
        e.surface = CSP_SURFACE_FLAT;
    } else {
        err = "surface type not implemented: " + tok[17];
        return false;
    }
    e.reflectivity = 1.0;
    P.elements.push_back(e);
    P.optic_of.push_back(tok[27]);
    return true;
}

int parse(const char* path, Parsed& P, std::string& err) {
    FILE* fp = std::fopen(path, "r");
    if (!fp) {
        err = std::string("failed to open system input file ") + path;
        return CSP_ERR_IO;
    }
    LineReader r(fp);
    int rc = CSP_OK;
    auto bad = [&](const std::string& m) {
        err = m;
        rc = CSP_ERR_PARSE;
    };
    const int c = std::fgetc(fp);
    if (c != '#') {
        bad("input file must start with '#'");
    } else {
        r.next();  // " SOLTRACE VERSION ... INPUT FILE"
        int bi = 0, count = 0;
        char shape = 'g';
        double sigma = 0, half = 0;
        std::sscanf(r.next(), "SUN\tPTSRC\t%d\tSHAPE\t%c\tSIGMA\t%lg\tHALFWIDTH\t%lg", &bi, &shape, &sigma, &half);
        P.sun_angle = sigma * 0.001;
        double X = 0, Y = 0, Z = 0, lat = 0, day = 0, hour = 0;
        std::sscanf(r.next(), "XYZ\t%lg\t%lg\t%lg\tUSELDH\t%d\tLDH\t%lg\t%lg\t%lg", &X, &Y, &Z, &bi, &lat, &day, &hour);
        P.sun[0] = X;
        P.sun[1] = Y;
        P.sun[2] = Z;
        std::sscanf(r.next(), "USER SHAPE DATA\t%d", &count);
        for (int i = 0; i < count; ++i) r.next();
        count = 0;
        std::sscanf(r.next(), "OPTICS LIST COUNT\t%d", &count);
        for (int i = 0; i < count && rc == CSP_OK; ++i) {
            const std::string head = r.next();
            if (head.compare(0, 12, "OPTICAL PAIR") != 0) {
                bad("expected OPTICAL PAIR, got: " + head);
                break;
            }
            std::string name = head.size() > 13 ? head.substr(13) : std::string();
            OpticSurface front, back;
            std::string e1, e2;
            read_optic_surface(r, &front, e1);  // the reference ignores these results
            read_optic_surface(r, &back, e2);
            P.optics[name] = front;
        }
        count = 0;
        if (rc == CSP_OK) std::sscanf(r.next(), "STAGE LIST COUNT\t%d", &count);
        for (int s = 0; s < count && rc == CSP_OK; ++s) {
            int virt = 0, multi = 1, n = 0, tr = 0;
            double sx, sy, sz, ax, ay, az, zr;
            std::sscanf(r.next(),
                        "STAGE\tXYZ\t%lg\t%lg\t%lg\tAIM\t%lg\t%lg\t%lg\tZROT\t%lg\tVIRTUAL\t%d\tMULTIHIT\t%d\t"
                        "ELEMENTS\t%d\tTRACETHROUGH\t%d",
                        &sx, &sy, &sz, &ax, &ay, &az, &zr, &virt, &multi, &n, &tr);
            r.next();  // stage name
            for (int i = 0; i < n; ++i) {
                std::string e;
                if (!read_element(r, P, e)) {
                    bad("error in element " + std::to_string(i) + ": " + e);
                    break;
                }
            }
        }
    }
    std::fclose(fp);
    return rc;
}

// ------------------------------------------------------------------------------ CSV writer ----
struct WriterState {
    uint64_t current = 1;
    int stage = 0;
};

inline bool is_marker(const float* r) { return r[1] == 0 && r[2] == 0 && r[3] == 0; }

// Advance the writer state over rays [b, e) without formatting.
void advance(const float* hits, uint64_t b, uint64_t e, WriterState& st) {
    for (uint64_t k = b * kMaxDepth; k < e * kMaxDepth; ++k) {
        const float* r = hits + 4 * k;
        if (is_marker(r)) {
            if (st.stage > 0) {
                st.current++;
                st.stage = 0;
            }
            continue;
        }
        if (st.stage < kMaxDepth) {
            st.stage++;
        } else {
            st.current++;
            st.stage = 1;
        }
    }
}

// A ray whose first interaction is the receiver (a stage-2 record in slot 1): light straight from
// the sun, which a staged SolTrace run never records (scripts/post_processing/clean_direct_sun.py:
// 6-18 drops the rows of every ray number with a stage-2 row and no stage-1 row; a ray's rows are
// its stage-0 sun point, its mirror interactions, then at most one receiver record, so that is a
// stage-2 record in slot 1).
inline bool direct_sun(const float* hits, uint64_t ray) { return hits[4 * (ray * kMaxDepth + 1)] == 2.0f; }

// longest row: a 20-digit ray number, four values of at most 16 characters, separators
constexpr size_t kMaxRowBytes = 20 + 4 * (1 + 16) + 1;

void format(const float* hits, uint64_t b, uint64_t e, WriterState st, bool staged, std::string& out) {
    out.resize((e - b) * 48 + 64 * kMaxRowBytes);  // about one row per ray; grown when short
    char* p = &out[0];
    char* end = p + out.size();
    for (uint64_t k = b * kMaxDepth; k < e * kMaxDepth; ++k) {
        if ((size_t)(end - p) < kMaxRowBytes) {
            const size_t used = (size_t)(p - out.data());
            out.resize(out.size() * 2);
            p = &out[0] + used;
            end = &out[0] + out.size();
        }
        const float* r = hits + 4 * k;
        if (is_marker(r)) {
            if (st.stage > 0) {
                st.current++;
                st.stage = 0;
            }
            continue;
        }
        if (st.stage >= kMaxDepth) {
            st.current++;
            st.stage = 0;
        }
        if (staged && direct_sun(hits, k / kMaxDepth)) {
            // the rows are dropped, the ray keeps its number (the state advances as if written)
            st.stage++;
            continue;
        }
        p = std::to_chars(p, end, st.current).ptr;
        for (int c = 0; c < 4; ++c) {
            *p++ = ',';
            p = format_g6(r[c], p, end);
        }
        *p++ = '\n';
        st.stage++;
    }
    out.resize((size_t)(p - out.data()));
}

}  // namespace

int write_hits_csv(const float* hits, uint64_t n, const char* path, bool staged, std::string& err) {
    FILE* fp = std::fopen(path, "wb");
    if (!fp) {
        err = std::string("could not open ") + path + " for writing";
        return CSP_ERR_IO;
    }
    const char* header = "number,stage,loc_x,loc_y,loc_z\n";
    std::fwrite(header, 1, std::strlen(header), fp);
    // batches of nt blocks: while the threads format batch i, this thread computes the start states
    // of batch i + 1 and writes batch i - 1
    const unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    const uint64_t block = 1u << 18;
    struct Batch {
        std::vector<WriterState> starts;
        std::vector<uint64_t> bb, ee;
        std::vector<std::string> bufs;
        std::vector<std::thread> th;
    } batch[2];
    WriterState st;
    auto plan = [&](Batch& B, uint64_t base) {
        B.starts.assign(nt, WriterState{});
        B.bb.assign(nt, 0);
        B.ee.assign(nt, 0);
        B.bufs.resize(nt);
        for (unsigned t = 0; t < nt; ++t) {
            B.bb[t] = std::min(n, base + t * block);
            B.ee[t] = std::min(n, B.bb[t] + block);
            B.starts[t] = st;
            advance(hits, B.bb[t], B.ee[t], st);
        }
    };
    auto launch = [&](Batch& B) {
        for (unsigned t = 0; t < nt; ++t)
            if (B.bb[t] < B.ee[t])
                B.th.emplace_back(format, hits, B.bb[t], B.ee[t], B.starts[t], staged, std::ref(B.bufs[t]));
    };
    auto join = [&](Batch& B) {
        for (auto& x : B.th) x.join();
        B.th.clear();
    };
    bool ok = true;
    auto write = [&](Batch& B) {
        for (unsigned t = 0; t < nt && ok; ++t)
            if (B.bb[t] < B.ee[t] && std::fwrite(B.bufs[t].data(), 1, B.bufs[t].size(), fp) != B.bufs[t].size())
                ok = false;
    };
    const uint64_t step = block * nt;
    if (n > 0) {
        plan(batch[0], 0);
        launch(batch[0]);
        for (uint64_t base = 0, i = 0;; base += step, ++i) {
            Batch& cur = batch[i & 1];
            Batch& nxt = batch[(i + 1) & 1];
            const bool more = base + step < n;
            if (more) plan(nxt, base + step);
            join(cur);
            if (more) launch(nxt);
            write(cur);
            if (!more) break;
            if (!ok) {
                join(nxt);
                break;
            }
        }
    }
    if (!ok) {
        std::fclose(fp);
        err = std::string("short write to ") + path;
        return CSP_ERR_IO;
    }
    if (std::fclose(fp) != 0) {
        err = std::string("could not close ") + path;
        return CSP_ERR_IO;
    }
    return CSP_OK;
}

// The CSV of compact records (csp_run_to_host_compact): blocks of rays are expanded back into their
// dense rows (sun-plane record, the ray's records, empty slots) and written by the dense writer's
// state machine and formatter, so the file is the one write_hits_csv makes from the dense buffer.
int write_compact_csv(const float* points, const uint8_t* counts, const float* records, uint64_t n, const char* path,
                      bool staged, std::string& err) {
    for (uint64_t r = 0; r < n; ++r)
        if (counts[r] >= kMaxDepth) {
            err = "ray " + std::to_string(r) + " has more than " + std::to_string(kMaxDepth - 1) + " records";
            return CSP_ERR_INVALID_ARGUMENT;
        }
    FILE* fp = std::fopen(path, "wb");
    if (!fp) {
        err = std::string("could not open ") + path + " for writing";
        return CSP_ERR_IO;
    }
    const char* header = "number,stage,loc_x,loc_y,loc_z\n";
    std::fwrite(header, 1, std::strlen(header), fp);
    const unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    const uint64_t block = 1u << 16;
    WriterState st;
    uint64_t rec = 0;  // first record of the next block
    // formatted blocks double-buffered: batch i is written by `writer` while batch i + 1 is built
    std::vector<std::string> bufs2[2] = {std::vector<std::string>(nt), std::vector<std::string>(nt)};
    std::vector<uint64_t> written_bb[2] = {std::vector<uint64_t>(nt), std::vector<uint64_t>(nt)};
    std::vector<uint64_t> written_ee[2] = {std::vector<uint64_t>(nt), std::vector<uint64_t>(nt)};
    std::thread writer;
    bool ok = true;
    std::vector<std::vector<float>> dense(nt);
    uint64_t batch_no = 0;
    for (uint64_t base = 0; base < n; base += block * nt, ++batch_no) {
        std::vector<std::string>& bufs = bufs2[batch_no & 1];
        std::vector<uint64_t> bb(nt), ee(nt), r0(nt);
        for (unsigned t = 0; t < nt; ++t) {
            bb[t] = std::min(n, base + t * block);
            ee[t] = std::min(n, bb[t] + block);
            r0[t] = rec;
            for (uint64_t r = bb[t]; r < ee[t]; ++r) rec += counts[r];
        }
        auto expand = [&](unsigned t) {
            std::vector<float>& d = dense[t];
            d.assign((ee[t] - bb[t]) * kMaxDepth * 4, 0.0f);
            uint64_t k = r0[t];
            for (uint64_t r = bb[t]; r < ee[t]; ++r) {
                float* row = d.data() + (r - bb[t]) * kMaxDepth * 4;
                row[1] = points[3 * r];
                row[2] = points[3 * r + 1];
                row[3] = points[3 * r + 2];
                for (uint32_t c = 0; c < counts[r]; ++c, ++k) std::memcpy(row + 4 * (1 + c), records + 4 * k, 16);
            }
        };
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; ++t)
            if (bb[t] < ee[t]) th.emplace_back(expand, t);
        for (auto& x : th) x.join();
        th.clear();
        std::vector<WriterState> starts(nt);
        for (unsigned t = 0; t < nt; ++t) {
            starts[t] = st;
            if (bb[t] < ee[t]) advance(dense[t].data(), 0, ee[t] - bb[t], st);
        }
        for (unsigned t = 0; t < nt; ++t)
            if (bb[t] < ee[t])
                th.emplace_back(format, dense[t].data(), 0, ee[t] - bb[t], starts[t], staged, std::ref(bufs[t]));
        for (auto& x : th) x.join();
        if (writer.joinable()) writer.join();  // the batch before is on disk
        if (!ok) break;
        written_bb[batch_no & 1] = bb;
        written_ee[batch_no & 1] = ee;
        writer = std::thread([&, slot = batch_no & 1] {
            for (unsigned t = 0; t < nt && ok; ++t)
                if (written_bb[slot][t] < written_ee[slot][t] &&
                    std::fwrite(bufs2[slot][t].data(), 1, bufs2[slot][t].size(), fp) != bufs2[slot][t].size())
                    ok = false;
        });
    }
    if (writer.joinable()) writer.join();
    if (!ok) {
        std::fclose(fp);
        err = std::string("short write to ") + path;
        return CSP_ERR_IO;
    }
    if (std::fclose(fp) != 0) {
        err = std::string("could not close ") + path;
        return CSP_ERR_IO;
    }
    return CSP_OK;
}

}  // namespace csp

extern "C" {

int csp_write_compact_csv(const float* points, const uint8_t* counts, const float* records, uint64_t num_rays,
                          const char* path, int flags) {
    if (!path || (num_rays && (!points || !counts))) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null argument");
    if (flags & ~CSP_OUT_STAGED) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "unknown output flags");
    uint64_t total = 0;
    for (uint64_t r = 0; r < num_rays; ++r) total += counts[r];
    if (total && !records) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null records");
    std::string err;
    const int rc = csp::write_compact_csv(points, counts, records, num_rays, path, (flags & CSP_OUT_STAGED) != 0, err);
    return rc ? csp::set_error(rc, err) : CSP_OK;
}

int csp_parse_stinput(const char* path, csp_element* out, uint32_t capacity, uint32_t* count, double* sun_dir,
                      double* sun_angle, int flags) {
    if (!path || !count) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null argument");
    csp::Parsed P;
    std::string err;
    int rc = csp::parse(path, P, err);
    if (rc) return csp::set_error(rc, err);
    if (flags & CSP_STINPUT_APPLY_OPTICS) {
        for (size_t i = 0; i < P.elements.size(); ++i) {
            auto it = P.optics.find(P.optic_of[i]);
            if (it == P.optics.end()) continue;
            P.elements[i].reflectivity = it->second.reflectivity;
            P.elements[i].slope_error = it->second.slope_mrad * 1e-3;
            P.elements[i].specularity_error = it->second.spec_mrad * 1e-3;
        }
    }
    *count = (uint32_t)P.elements.size();
    if (sun_dir) {
        sun_dir[0] = P.sun[0];
        sun_dir[1] = P.sun[1];
        sun_dir[2] = P.sun[2];
    }
    if (sun_angle) *sun_angle = P.sun_angle;
    if (out) {
        if (capacity < P.elements.size()) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "output capacity too small");
        std::copy(P.elements.begin(), P.elements.end(), out);
    }
    return CSP_OK;
}

int csp_read_stinput(csp_handle h, const char* path, int flags) {
    if (!h) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null handle");
    uint32_t n = 0;
    double sun[3], angle = 0;
    int rc = csp_parse_stinput(path, nullptr, 0, &n, sun, &angle, flags);
    if (rc) return rc;
    std::vector<csp_element> el(n);
    rc = csp_parse_stinput(path, el.data(), n, &n, sun, &angle, flags);
    if (rc) return rc;
    csp::System* s = reinterpret_cast<csp::System*>(h);
    s->elements.insert(s->elements.end(), el.begin(), el.end());
    s->sun_dir[0] = sun[0];
    s->sun_dir[1] = sun[1];
    s->sun_dir[2] = sun[2];
    s->sun_shape = CSP_SUN_PILLBOX;
    s->sun_param = angle;
    return CSP_OK;
}

int csp_write_hits_csv_ex(const float* hits, uint64_t num_rays, const char* path, int flags) {
    if (!path || (!hits && num_rays)) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null argument");
    if (flags & ~CSP_OUT_STAGED) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "unknown output flags");
    std::string err;
    const int rc = csp::write_hits_csv(hits, num_rays, path, (flags & CSP_OUT_STAGED) != 0, err);
    return rc ? csp::set_error(rc, err) : CSP_OK;
}

int csp_write_hits_csv(const float* hits, uint64_t num_rays, const char* path) {
    return csp_write_hits_csv_ex(hits, num_rays, path, 0);
}

int csp_write_output(csp_handle h, const char* path) { return csp_write_output_ex(h, path, 0); }

int csp_write_output_ex(csp_handle h, const char* path, int flags) {
    if (!h) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null handle");
    csp::System* s = reinterpret_cast<csp::System*>(h);
    if (!s->initialized) return csp::set_error(CSP_ERR_STATE, "write_output before initialize()");
    std::vector<float> host;
    try {
        host.resize((size_t)s->num_rays * csp::kMaxDepth * 4);
    } catch (...) {
        return csp::set_error(CSP_ERR_OUT_OF_MEMORY, "host buffer for the hit records");
    }
    int rc = csp_copy_hits(h, host.data(), nullptr, 0, s->num_rays);
    if (rc) return rc;
    return csp_write_hits_csv_ex(host.data(), s->num_rays, path, flags);
}

}  // extern "C"
