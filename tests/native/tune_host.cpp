// Host build of the tuning cache logic (prime-gap_gb300/csrc/pg_tuning.h) for
// CPU tests: class keys, line format, file merge across devices.
#include <cstring>
#include <map>
#include <string>

#include "pg_tuning.h"

extern "C" {

// Sets (device, cls) to t in the file, keeping every other entry.
int th_put(const char *path, const char *device, const char *cls, const pgs_tuning *t, double ms_default,
           double ms_tuned) {
    std::map<std::string, pgt::Entry> m;
    pgt::load(path, device, m);
    pgt::Entry e;
    e.t = *t;
    e.ms_default = ms_default;
    e.ms_tuned = ms_tuned;
    m[cls] = e;
    return pgt::save(path, device, m);
}

// 1 and the entry when the file has (device, cls); 0 when not; -1 unreadable.
int th_get(const char *path, const char *device, const char *cls, pgs_tuning *out, double *ms2) {
    std::map<std::string, pgt::Entry> m;
    if (pgt::load(path, device, m) < 0) return -1;
    auto it = m.find(cls);
    if (it == m.end()) return 0;
    *out = it->second.t;
    ms2[0] = it->second.ms_default;
    ms2[1] = it->second.ms_tuned;
    return 1;
}

// 1 when the line parses into a valid entry.
int th_parse(const char *line, pgs_tuning *out) {
    std::string dev, cls;
    pgt::Entry e;
    if (!pgt::parse_line(line, dev, cls, e)) return 0;
    *out = e.t;
    return 1;
}

int th_class(const pgs_job *job, char *buf, size_t cap) {
    const std::string c = pgt::tuning_class(*job);
    if (c.size() + 1 > cap) return -1;
    memcpy(buf, c.c_str(), c.size() + 1);
    return (int)c.size();
}

}
