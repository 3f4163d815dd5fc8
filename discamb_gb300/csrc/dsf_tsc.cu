// .tsc reader: tabulated atomic form factors as written for olex2 / NoSpherA2
// (the reference's tsc_io::read_tsc, src/IO/tsc_io.cpp:60-125, and
// TscFileBasedSfCalculator, src/Scattering/TscFileBasedSfCalculator.cpp:17-123).
//
// Format: header lines up to "DATA:" ("SCATTERERS: label ..." names the atom
// columns), then one line per reflection h' of the symmetry-expanded set:
// "h k l re,im re,im ..." with one complex value per scatterer.  Lines with
// another number of fields are skipped, as the reference does.  The reader
// parses straight into flat arrays (several threads over line-aligned
// chunks) instead of a std::map, and dsf_structure_create_tsc expands the
// table to the structure's reflections and operations (h' = h R, the lookup
// of ConstFormFactorCalculationsManager, src/Scattering/
// ConstFormFactorCalculationsManager.cpp:34-102) on the host into complex64
// and hands it to the device-table constructor.
#include "../../include/dsf_gb300.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

struct TscTable {
    int n_atoms = 0;
    std::vector<int> hkl;        // [rows][3]
    std::vector<double> values;  // [rows][n_atoms][2]
};

bool read_file(const char *path, std::string &buf)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (n < 0) {
        std::fclose(f);
        return false;
    }
    buf.resize((size_t)n);
    const size_t got = n ? std::fread(&buf[0], 1, (size_t)n, f) : 0;
    std::fclose(f);
    return got == (size_t)n;
}

// one data line [p, e): 3 integers and n complex "re,im" fields separated by blanks; false if it has another form
bool parse_line(const char *p, const char *e, int n, int *h, double *v)
{
    auto skip = [&](const char *q) {
        while (q < e && (*q == ' ' || *q == '\t' || *q == '\r')) q++;
        return q;
    };
    const char *q = skip(p);
    for (int j = 0; j < 3; j++) {
        if (q >= e) return false;
        char *end;
        const long x = std::strtol(q, &end, 10);
        if (end == q || end > e) return false;
        h[j] = (int)x;
        q = skip(end);
    }
    for (int a = 0; a < n; a++) {
        if (q >= e) return false;
        char *end;
        v[2 * a] = std::strtod(q, &end);
        if (end == q || end >= e || *end != ',') return false;
        q = end + 1;
        v[2 * a + 1] = std::strtod(q, &end);
        if (end == q || end > e) return false;
        q = skip(end);
    }
    return q >= e;  // nothing after the last field
}

int parse_tsc(const char *path, TscTable &t, std::string &err)
{
    std::string buf;
    if (!read_file(path, buf)) {
        err = std::string("cannot read tsc file ") + path;
        return DSF_ERR_ARGUMENT;
    }
    // header
    size_t pos = 0, data = std::string::npos;
    std::vector<std::string> labels;
    while (pos < buf.size()) {
        size_t eol = buf.find('\n', pos);
        if (eol == std::string::npos) eol = buf.size();
        const std::string line = buf.substr(pos, eol - pos);
        pos = eol + 1;
        size_t a = line.find_first_not_of(" \t\r");
        if (a == std::string::npos) continue;
        if (line.compare(a, 5, "DATA:") == 0) {
            data = pos;
            break;
        }
        if (line.compare(a, 11, "SCATTERERS:") == 0) {
            size_t q = a + 11;
            while (q < line.size()) {
                q = line.find_first_not_of(" \t\r", q);
                if (q == std::string::npos) break;
                size_t r = line.find_first_of(" \t\r", q);
                if (r == std::string::npos) r = line.size();
                labels.push_back(line.substr(q, r - q));
                q = r;
            }
        }
    }
    if (data == std::string::npos) {
        err = "tsc file has no DATA: section";
        return DSF_ERR_ARGUMENT;
    }
    const int n = (int)labels.size();
    if (n < 1) {
        err = "tsc file lists no scatterers";
        return DSF_ERR_ARGUMENT;
    }
    t.n_atoms = n;
    // line-aligned chunks, parsed in parallel, concatenated in file order
    const size_t len = buf.size() - data;
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (len < (1u << 20)) nt = 1;
    std::vector<size_t> cut(nt + 1, data);
    cut[nt] = buf.size();
    for (unsigned k = 1; k < nt; k++) {
        size_t c = data + len * k / nt;
        const size_t nl = buf.find('\n', c);
        cut[k] = nl == std::string::npos ? buf.size() : nl + 1;
        if (cut[k] < cut[k - 1]) cut[k] = cut[k - 1];
    }
    std::vector<std::vector<int> > hk(nt);
    std::vector<std::vector<double> > va(nt);
    auto work = [&](unsigned k) {
        const char *p = buf.data() + cut[k], *end = buf.data() + cut[k + 1];
        std::vector<double> v(2 * (size_t)n);
        int h[3];
        while (p < end) {
            const char *e = (const char *)std::memchr(p, '\n', (size_t)(end - p));
            if (!e) e = end;
            if (parse_line(p, e, n, h, v.data())) {
                hk[k].insert(hk[k].end(), h, h + 3);
                va[k].insert(va[k].end(), v.begin(), v.end());
            }
            p = e + 1;
        }
    };
    std::vector<std::thread> th;
    for (unsigned k = 1; k < nt; k++) th.emplace_back(work, k);
    work(0);
    for (auto &x : th) x.join();
    for (unsigned k = 0; k < nt; k++) {
        t.hkl.insert(t.hkl.end(), hk[k].begin(), hk[k].end());
        t.values.insert(t.values.end(), va[k].begin(), va[k].end());
    }
    return DSF_OK;
}

inline uint64_t key3(int h, int k, int l)
{
    return ((uint64_t)(uint32_t)(h + (1 << 20)) << 42) | ((uint64_t)(uint32_t)(k + (1 << 20)) << 21) |
           (uint64_t)(uint32_t)(l + (1 << 20));
}

}  // namespace

namespace dsf {

// the table of a .tsc file at h' = h R for the reflections hkl and operations rot ([ns][9]), complex64
// [n_hkl][ns][n_atoms]; DSF_ERR_ARGUMENT (with err) for an unreadable file, another scatterer count or a missing h'
int tsc_expand(const char *path, int n_atoms, int n_hkl, const int *hkl, int ns, const int *rot,
               std::vector<float> &tab, std::string &err)
{
    TscTable t;
    int rc = parse_tsc(path, t, err);
    if (rc) return rc;
    if (t.n_atoms != n_atoms) {
        err = "tsc file lists " + std::to_string(t.n_atoms) + " scatterers, the structure has " + std::to_string(n_atoms);
        return DSF_ERR_ARGUMENT;
    }
    const int rows = (int)(t.hkl.size() / 3), n = n_atoms;
    std::unordered_map<uint64_t, int> row_of;
    row_of.reserve((size_t)rows * 2);
    for (int r = 0; r < rows; r++) row_of[key3(t.hkl[3 * r], t.hkl[3 * r + 1], t.hkl[3 * r + 2])] = r;
    tab.assign(2 * (size_t)n_hkl * ns * n, 0.0f);
    for (int i = 0; i < n_hkl; i++)
        for (int s = 0; s < ns; s++) {
            const int *R = rot + 9 * s;
            int hp[3];
            for (int j = 0; j < 3; j++)
                hp[j] = hkl[3 * i] * R[0 * 3 + j] + hkl[3 * i + 1] * R[1 * 3 + j] + hkl[3 * i + 2] * R[2 * 3 + j];
            auto it = row_of.find(key3(hp[0], hp[1], hp[2]));
            if (it == row_of.end()) {
                err = "tsc file has no form factors for " + std::to_string(hp[0]) + " " + std::to_string(hp[1]) + " " +
                      std::to_string(hp[2]);
                return DSF_ERR_ARGUMENT;
            }
            const double *v = t.values.data() + 2 * (size_t)it->second * n;
            float *d = tab.data() + 2 * ((size_t)i * ns + s) * n;
            for (int a = 0; a < 2 * n; a++) d[a] = (float)v[a];
        }
    return DSF_OK;
}

}  // namespace dsf

extern "C" {

int dsf_tsc_load(const char *path, int *n_atoms, int *n_rows, int *hkl, double *values, int capacity_rows)
{
    if (!path || !n_atoms || !n_rows) return DSF_ERR_ARGUMENT;
    TscTable t;
    std::string err;
    int rc = parse_tsc(path, t, err);
    if (rc) return rc;
    const int rows = (int)(t.hkl.size() / 3);
    *n_atoms = t.n_atoms;
    *n_rows = rows;
    if (!hkl || !values) return DSF_OK;
    if (capacity_rows < rows) return DSF_ERR_ARGUMENT;
    std::memcpy(hkl, t.hkl.data(), sizeof(int) * t.hkl.size());
    std::memcpy(values, t.values.data(), sizeof(double) * t.values.size());
    return DSF_OK;
}

}  // extern "C"
