// Event averaging of the HBT correlation files over many event folders
// (the reference's ebe_scripts/average_event_HBT_correlation_function.py):
// the folders are the entries of the working folder whose names start with
// "UrQMD", in directory order (Python's glob order); the files are the
// "HBT*" files of the first folder's UrQMD_results; each output file is the
// element-wise sum over the folders of the numbers in that file, started
// from 0 * (the first folder's numbers) and divided by the folder count,
// written with "%.10e" and two blanks between columns (numpy.savetxt).
//
// Here, file by file, the folders are parsed on all host threads (chunks of
// one folder per thread, std::from_chars) and added in the script's folder
// order, so each element is the script's value exactly; the rows are then
// formatted in parallel.
#include <dirent.h>
#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "SampleSource.h"
#include "TextNumbers.h"
#include "hbt_host.h"

namespace {

bool read_all(const std::string &path, std::string &out) {
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return false;
    out.clear();
    char buf[1 << 16];
    size_t got;
    while ((got = fread(buf, 1, sizeof(buf), f)) > 0) out.append(buf, got);
    fclose(f);
    return true;
}

// numpy.loadtxt of a whitespace-separated table ('#' comments, blank lines
// skipped); false when rows differ in length or a token is not a number.
bool load_table(const std::string &text, std::vector<double> &vals, long &rows, int &cols) {
    vals.clear();
    rows = 0;
    cols = -1;
    const char *p = text.data(), *end = p + text.size();
    double v[64];
    while (p < end) {
        const char *nl = static_cast<const char *>(memchr(p, '\n', end - p));
        const char *le = nl ? nl : end;
        const char *hash = static_cast<const char *>(memchr(p, '#', le - p));
        const char *ce = hash ? hash : le;
        const char *q = p;
        while (q < ce && hbt::is_space(*q)) q++;
        if (q < ce) {
            // count the tokens, then parse them all
            int ntok = 0;
            for (const char *t = q; t < ce;) {
                while (t < ce && hbt::is_space(*t)) t++;
                if (t >= ce) break;
                ntok++;
                while (t < ce && !hbt::is_space(*t)) t++;
            }
            if (ntok > 64 || (cols >= 0 && ntok != cols)) return false;
            if (hbt::parse_span(q, ce, v, ntok) != ntok) return false;
            cols = ntok;
            vals.insert(vals.end(), v, v + ntok);
            rows++;
        }
        p = le + 1;
    }
    return cols > 0;
}

// Python's "%.10e" (a NaN prints as "nan" whatever its sign bit).
char *put_py_e10(char *p, double v) {
    if (std::isnan(v)) {
        memcpy(p, "nan", 3);
        return p + 3;
    }
    return hbt::put_sci(p, v, 10);
}

std::vector<std::string> list_dir(const std::string &dir) {
    std::vector<std::string> out;
    DIR *d = opendir(dir.c_str());
    if (!d) return out;
    while (dirent *e = readdir(d)) out.push_back(e->d_name);
    closedir(d);
    return out;
}

bool starts_with(const std::string &s, const char *prefix) {
    return s.compare(0, strlen(prefix), prefix) == 0;
}

}  // namespace

extern "C" int hbt_host_average_events(const char *working_folder, const char *avg_folder,
                                       int32_t threads) {
    try {
        if (!working_folder || !avg_folder) return -1;
        const std::string work(working_folder), avg(avg_folder);
        std::vector<std::string> folders;
        for (const std::string &n : list_dir(work))
            if (starts_with(n, "UrQMD")) folders.push_back(work + "/" + n);
        if (folders.empty()) throw std::runtime_error("no UrQMD* event folders in " + work);
        const std::string sub = "/UrQMD_results";
        std::vector<std::string> files;
        for (const std::string &n : list_dir(folders[0] + sub))
            if (starts_with(n, "HBT")) files.push_back(n);
        mkdir(avg.c_str(), 0755);
        const int T = threads > 0 ? threads
                                  : std::max(1, static_cast<int>(std::thread::hardware_concurrency()));
        const double nev = static_cast<double>(folders.size());
        std::vector<std::string> text(T);
        std::vector<std::vector<double>> vals(T);
        std::vector<long> rows_of(T);
        std::vector<int> cols_of(T);
        std::vector<double> acc;
        for (const std::string &name : files) {
            // folders in chunks of T parsed in parallel, added in folder order
            long rows = 0;
            int cols = 0;
            for (size_t c0 = 0; c0 < folders.size(); c0 += T) {
                const long nc = static_cast<long>(std::min(folders.size() - c0, (size_t)T));
                std::atomic<bool> bad(false);
                hbt::parallel_ranges(nc, T, 1, [&](long lo, long hi) {
                    for (long k = lo; k < hi; k++) {
                        const std::string path = folders[c0 + k] + sub + "/" + name;
                        if (!read_all(path, text[k]) ||
                            !load_table(text[k], vals[k], rows_of[k], cols_of[k]))
                            bad = true;
                    }
                });
                if (bad) throw std::runtime_error("cannot read " + name + " in every folder, or "
                                                  "it is not a table of numbers");
                for (long k = 0; k < nc; k++) {
                    if (c0 == 0 && k == 0) {
                        rows = rows_of[0];
                        cols = cols_of[0];
                        acc.resize(vals[0].size());
                        for (size_t i = 0; i < acc.size(); i++) acc[i] = 0.0 * vals[0][i];
                    }
                    if (rows_of[k] != rows || cols_of[k] != cols)
                        throw std::runtime_error(name + ": tables differ in shape between folders");
                    const std::vector<double> &v = vals[k];
                    for (size_t i = 0; i < acc.size(); i++) acc[i] += v[i];
                }
            }
            // format row ranges in parallel, write in order
            std::vector<std::string> parts(T);
            const long per = (rows + T - 1) / T;
            hbt::parallel_ranges(T, T, 1, [&](long lo, long hi) {
                for (long t = lo; t < hi; t++) {
                    const long r0 = t * per, r1 = std::min(rows, r0 + per);
                    std::string &out = parts[t];
                    out.assign(static_cast<size_t>(std::max(0L, r1 - r0)) * cols * 24 + 16, '\0');
                    char *o = &out[0];
                    for (long r = r0; r < r1; r++) {
                        for (int c = 0; c < cols; c++) {
                            if (c > 0) {
                                *o++ = ' ';
                                *o++ = ' ';
                            }
                            o = put_py_e10(o, acc[r * cols + c] / nev);
                        }
                        *o++ = '\n';
                    }
                    out.resize(o - out.data());
                }
            });
            FILE *fo = fopen((avg + "/" + name).c_str(), "w");
            if (!fo) throw std::runtime_error("cannot write " + avg + "/" + name);
            bool ok = true;
            for (const std::string &part : parts)
                ok = ok && fwrite(part.data(), 1, part.size(), fo) == part.size();
            ok = (fclose(fo) == 0) && ok;
            if (!ok) throw std::runtime_error("cannot write " + avg + "/" + name);
        }
        return static_cast<int>(files.size());
    } catch (const std::exception &e) {
        fprintf(stderr, "error: %s\n", e.what());
        return -1;
    }
}
