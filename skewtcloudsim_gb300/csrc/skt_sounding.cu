// Sounding ingestion, host code: the radiosonde readers and the column interpolation of
// readTable (Game/readTable.cpp:27-474) with the meteorological formulas it calls
// (Engine/source/math/meteoformulas.cpp:8-22,184-202; constants Engine/include/math/constants.hpp).
//
// Bit-exact with the reference on the same host: every value goes through the same float
// operations in the same order (this file is compiled without FP contraction), std::stof for the
// text, and the C library's expf/powf/sinf/cosf. The DWD reader keeps the reference's stream
// search (fixed-size probes on a std::stringstream) because that search decides which rows of an
// ascent are read. The zip container is the caller's (skt_archive_read_fn).
#include "skt_internal.cuh"

#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <sstream>
#include <string>
#include <vector>

namespace {

// Engine/include/math/constants.hpp:9,10,11,15,32
constexpr float kRsd = 287.0528f;
constexpr float kRsw = 461.5f;
constexpr float kE = kRsd / kRsw;
constexpr float kCpd = 1003.5f;
constexpr float kPi = 3.14159265359f;

constexpr long kProbe = 100000;  // byte stride of the DWD date search (Game/readTable.cpp:228,235)

struct Columns {
    std::vector<float> altitude, pressure, temperature, dew, speed, dir;
};

skt_status bad(const std::string& msg) { return skt::report(nullptr, SKT_INVALID_ARG, msg.c_str()); }

// std::stof: leading white space, the longest number prefix; no number or out of range is an error
bool parse_float(const std::string& w, float* v) {
    errno = 0;
    char* end = nullptr;
    const float f = std::strtof(w.c_str(), &end);
    if (end == w.c_str() || errno == ERANGE) return false;
    *v = f;
    return true;
}

// A KNMI attribute token: the value after a `prefix`-character name, less its closing quote.
bool attr_value(const std::string& w, size_t prefix, float* v) {
    if (w.size() <= prefix) return false;
    return parse_float(w.substr(prefix, w.size() - prefix - 1), v);
}

bool read_member(skt_archive_read_fn rd, void* ctx, const std::string& name, std::string* out) {
    const long long n = rd(ctx, name.c_str(), nullptr, 0);
    if (n < 0) return false;
    out->assign((size_t)n, '\0');
    return n == 0 || rd(ctx, name.c_str(), &(*out)[0], (size_t)n) == n;
}

skt_status publish(const Columns& c, size_t n, skt_sounding* out) {
    for (const std::vector<float>* v : {&c.altitude, &c.pressure, &c.temperature, &c.dew, &c.speed, &c.dir})
        if (v->size() < n) return bad("sounding columns of unequal length (a row misses a value)");
    if (n == 0) return bad("the sounding has no rows");
    float* blk = static_cast<float*>(std::malloc(6 * n * sizeof(float)));
    if (!blk) return skt::report(nullptr, SKT_OUT_OF_MEMORY, "sounding allocation failed");
    float** dst[6] = {&out->altitude, &out->pressure, &out->temperature, &out->dew_point, &out->wind_speed, &out->wind_dir};
    const std::vector<float>* src[6] = {&c.altitude, &c.pressure, &c.temperature, &c.dew, &c.speed, &c.dir};
    for (int k = 0; k < 6; k++) {
        *dst[k] = blk + k * n;
        std::memcpy(*dst[k], src[k]->data(), n * sizeof(float));
    }
    out->n = n;
    return SKT_OK;
}

void clear(skt_sounding* s) {
    s->n = 0;
    s->altitude = s->pressure = s->temperature = s->dew_point = s->wind_speed = s->wind_dir = nullptr;
}

// lerpEnvValue (Game/readTable.cpp:356-362)
float lerp_height(float h1, float h2, float hc, float v1, float v2) {
    if (hc == h1) return v1;
    if (hc == h2) return v2;
    const float t = (hc - h1) / (h2 - h1);
    return v1 + t * (v2 - v1);
}

// es, ws (Engine/source/math/meteoformulas.cpp:8-22): hPa, kg/kg
float sat_mixing_ratio(float t_c, float p_hpa) {
    const float es = 0.61078f * expf((17.27f * t_c) / (t_c + 237.3f)) * 10.0f;
    return (kE * es) / (p_hpa - es);
}

}  // namespace

extern "C" {

skt_status skt_sounding_read_knmi(skt_archive_read_fn rd, void* ctx, skt_sounding* out) {
    if (!rd || !out) return bad("null argument");
    clear(out);
    std::string text;
    if (!read_member(rd, ctx, "SynchronizedSoundingData.xml", &text))
        return bad("the archive has no SynchronizedSoundingData.xml");
    Columns c;
    std::istringstream s(text);
    std::string line, word;
    std::getline(s, line);  // the first line holds no row
    size_t lines = 0;
    while (std::getline(s, line)) {
        std::istringstream ts(line);
        for (int tok = 0; ts >> word; tok++) {
            float v = 0.0f;
            bool ok = true;
            switch (tok) {
                case 4: ok = attr_value(word, 10, &v); c.pressure.push_back(v); break;
                case 5: ok = attr_value(word, 13, &v); c.temperature.push_back(v - 273.15f); break;
                case 6: {  // relative humidity to dew point, with the temperature of row `lines`
                    ok = attr_value(word, 10, &v);
                    if (ok && lines >= c.temperature.size()) return bad("KNMI: humidity before its temperature");
                    const float t = ok ? c.temperature[lines] : 0.0f;
                    c.dew.push_back(t - ((100 - v) * 0.2f) * ((t + 273.15f) * 0.01f));
                    break;
                }
                case 7: ok = attr_value(word, 9, &v); c.dir.push_back(v); break;
                case 8: ok = attr_value(word, 11, &v); c.speed.push_back(v); break;
                default:
                    if (word.compare(0, 8, "Altitude") == 0) {
                        ok = attr_value(word, 10, &v);
                        c.altitude.push_back(v);
                    }
                    break;
            }
            if (!ok) return bad("KNMI: unreadable value '" + word + "' on row " + std::to_string(lines));
        }
        lines++;
    }
    if (lines < 2) return bad("KNMI: no rows");
    return publish(c, lines - 1, out);
}

skt_status skt_sounding_read_dwd(const char* archive_name, skt_archive_read_fn rd, void* ctx, skt_sounding* out) {
    if (!archive_name || !rd || !out) return bad("null argument");
    clear(out);
    // the station number: the third '_'-separated field of the archive name
    std::string station;
    {
        std::istringstream s(archive_name);
        std::string f;
        for (int k = 0; std::getline(s, f, '_'); k++)
            if (k == 2) { station = f; break; }
    }
    // the ascents the archive holds: field 1 of each line after the first, less its hour
    std::vector<std::string> dates;
    {
        const std::string name = "Metadaten_Sekunde_Aero_" + station + ".txt";
        std::string meta;
        if (!read_member(rd, ctx, name, &meta)) return bad("DWD: the archive has no " + name);
        std::istringstream s(meta);
        std::string line, f;
        std::getline(s, line);
        while (std::getline(s, line)) {
            std::istringstream fs(line);
            for (int k = 0; std::getline(fs, f, ';'); k++) {
                if (k == 1) {
                    if (f.size() < 2) return bad("DWD: short date field in " + name);
                    dates.push_back(f.substr(0, f.size() - 2));
                } else if (k == 8) {  // the station's ground temperature: read (and checked) but unused
                    float v;
                    if (!parse_float(f, &v)) return bad("DWD: unreadable ground temperature '" + f + "'");
                    break;
                }
            }
        }
    }
    if (dates.size() < 162) return bad("DWD: fewer than 162 ascents listed (the reference reads ascent 161)");
    const std::string target = dates[161] + "12";
    const std::string name = "produkt_sec_aero_" + dates.front() + "_" + dates.back() + "_" + station + ".txt";
    std::string prod;
    if (!read_member(rd, ctx, name, &prod)) return bad("DWD: the archive has no " + name);

    std::stringstream s(prod);
    std::string line, f;
    const std::string not_found = "DWD: could not find date " + target;
    // coarse search: look at one whole line per probe; on a hit, go back one probe and scan
    for (bool hit = false; !hit;) {
        std::getline(s, line);  // the rest of the line the stream is in (the header at first)
        std::getline(s, line);
        std::istringstream fs(line);
        for (int k = 0; std::getline(fs, f, ';'); k++) {
            if (k != 1) continue;
            if (f == target) {
                s.seekg(-kProbe, std::ios::cur);
                if (s.fail()) s.clear();
                hit = true;
                std::getline(s, line);
            } else {
                s.seekg(kProbe, std::ios::cur);
            }
            break;
        }
        if (s.tellg() == -1) return bad(not_found);
    }
    // scan: the rows from the first line of the target date to the next line of another date
    Columns c;
    size_t rows = 0;
    bool in_block = false, done = false;
    while (std::getline(s, line) && !done) {
        std::istringstream fs(line);
        int k = 0;
        while (std::getline(fs, f, ';')) {
            if (!in_block) {
                if (k == 1 && f == target) {
                    in_block = true;
                    k--;
                }
                k++;
            }
            if (in_block) {
                float v = 0.0f;
                bool ok = true;
                switch (k) {
                    case 1:
                        if (f != target) {
                            in_block = false;
                            done = true;
                        }
                        break;
                    case 6: ok = parse_float(f, &v); c.altitude.push_back(v); break;
                    case 7: ok = parse_float(f, &v); c.pressure.push_back(v); break;
                    case 8: ok = parse_float(f, &v); c.temperature.push_back(v); break;
                    case 10: ok = parse_float(f, &v); c.dew.push_back(v); break;
                    case 11: ok = parse_float(f, &v); c.speed.push_back(v); break;
                    case 12: ok = parse_float(f, &v); c.dir.push_back(v); break;
                    default: break;
                }
                if (!ok) return bad("DWD: unreadable value '" + f + "' in field " + std::to_string(k));
                k++;
            }
        }
        if (in_block) rows++;
        if (s.tellg() == -1) return bad(not_found);
    }
    return publish(c, rows, out);
}

void skt_sounding_free(skt_sounding* s) {
    if (!s) return;
    std::free(s->altitude);
    clear(s);
}

skt_status skt_sounding_to_init(const skt_sounding* s, const skt_grid_desc* grid, float* theta, float* vel_aos3,
                                float* qv, float* ground_T, float* ground_p, float* p3d, float* p_column) {
    if (!s || !grid || !theta || !vel_aos3 || !qv || !ground_T || !ground_p || !p3d || !p_column) return bad("null argument");
    if (s->n == 0 || !s->altitude || !s->pressure || !s->temperature || !s->dew_point || !s->wind_speed || !s->wind_dir)
        return bad("empty sounding");
    const int X = grid->nx, Y = grid->ny, Z = grid->nz;
    const float vox = grid->voxel;
    if (X < 1 || Y < 1 || Z < 1 || !(vox > 0.0f) || (long long)X * Y * Z >= (1ll << 31)) return bad("invalid grid");
    const float* alt = s->altitude;
    const size_t n = s->n;
    const float h0 = alt[0];

    // level pressures and temperatures at heights y = 0, voxel, 2 voxel, ... (a float running sum)
    std::vector<int> row(Y, 0);
    std::vector<float> p_lev(Y, 0.0f), t_lev(Y, 0.0f);
    int j = 0;
    const float top = (float)Y * vox;
    for (float y = 0; y < top && j < Y; y += vox, j++) {
        const float h = y + h0;
        size_t i = 0;
        while (i < n && !(h <= alt[i])) i++;
        if (i == n) return bad("the sounding ends below the grid top (level " + std::to_string(j) + ")");
        const size_t pi = i == 0 ? 0 : i - 1;
        p_lev[j] = lerp_height(alt[pi] - h0, alt[i] - h0, y, s->pressure[pi], s->pressure[i]);
        t_lev[j] = lerp_height(alt[pi] - h0, alt[i] - h0, y, s->temperature[pi], s->temperature[i]);
        row[j] = (int)i;
    }
    if (j < Y) return bad("the level heights reach the grid top early (voxel too small for a float sum)");
    // potential temperature relative to the first row's pressure (getPotentialTempArray)
    const float p0 = s->pressure[0];
    std::vector<float> th_lev(Y), u_lev(Y), w_lev(Y), ps_lev(Y), qv_lev(Y);
    for (int k = 0; k < Y; k++) th_lev[k] = ((t_lev[k] + 273.15f) * powf(p0 / p_lev[k], kRsd / kCpd) - 273.15f) + 273.15f;
    for (int k = 0; k < Y; k++) {
        const int i = row[k];
        const int pi = i == 0 ? 0 : i - 1;
        const int pk = k == 0 ? 0 : k - 1;
        const float ang = (s->wind_dir[i] - 180.0f) * (kPi / 180.0f);
        u_lev[k] = sinf(ang) * s->wind_speed[i];
        w_lev[k] = cosf(ang) * s->wind_speed[i];
        const float hk = k * vox;
        ps_lev[k] = lerp_height(alt[pi] - h0, alt[i] - h0, hk, p_lev[pk], p_lev[k]);
        qv_lev[k] = sat_mixing_ratio(lerp_height(alt[pi] - h0, alt[i] - h0, hk, s->dew_point[pi], s->dew_point[i]), ps_lev[k]);
    }
    // every column a copy; velocities averaged with the next cell (clamped) onto the MAC faces:
    // columns are uniform, so x and z neighbours hold the same level values
    const size_t XY = (size_t)X * Y;
    for (int z = 0; z < Z; z++)
        for (int y = 0; y < Y; y++) {
            const float u = (u_lev[y] + u_lev[y]) / 2.0f;
            const float v = 0.0f;  // (0 + 0) / 2 with the cell above
            const float w = (w_lev[y] + w_lev[y]) / 2.0f;
            for (int x = 0; x < X; x++) {
                const size_t idx = x + y * (size_t)X + z * XY;
                theta[idx] = th_lev[y];
                qv[idx] = qv_lev[y];
                p3d[idx] = ps_lev[y];
                vel_aos3[3 * idx + 0] = u;
                vel_aos3[3 * idx + 1] = v;
                vel_aos3[3 * idx + 2] = w;
            }
        }
    const float gT = s->temperature[0] + 273.15f;
    for (size_t k = 0; k < (size_t)X * Z; k++) {
        ground_T[k] = gT;
        ground_p[k] = p0;
    }
    for (int k = 0; k < Y; k++) p_column[k] = p_lev[k];
    return SKT_OK;
}

}  // extern "C"
