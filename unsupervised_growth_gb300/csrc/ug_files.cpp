// The reference's directory formats on top of the C ABI: read_network_state
// (NetworkGrowthSimulator.cpp:1943-2020) and the writers it reads back
// (write_full_network_state :18552-18593, write_network_topology :18294-18310,
// the appended records and the jitter file).  Little-endian 4-byte ints and
// 8-byte doubles, laid out field by field as those writers lay them out; the
// two parameter files are the libconfig text of ConfigurationNetworkGrowth /
// ConfigurationNetworkTopology, of which this parser reads the subset they use
// (groups of scalar settings, '=' or ':', quoted strings, comments).
#include "ugrowth.h"
#include "ug_philox.cuh"
#include "ug_topology.h"

#include <sys/stat.h>

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <numeric>
#include <string>
#include <vector>


namespace {

ug_status ferr(ug_status s, const std::string& msg)
{
    ug_set_last_error(msg);
    return s;
}

#define UG_FTRY(call)                     \
    do {                                  \
        ug_status s_ = (call);            \
        if (s_ != UG_OK) return s_;       \
    } while (0)

// ---------------------------------------------------------------- binary I/O
class In {
public:
    explicit In(const std::string& path) : path_(path), f_(path, std::ios::binary) {}
    bool ok() const { return (bool)f_; }
    template <class T>
    bool get(T& v) { return (bool)f_.read(reinterpret_cast<char*>(&v), sizeof(T)); }
    template <class T>
    bool get(std::vector<T>& v, size_t n)
    {
        v.resize(n);
        return n == 0 || (bool)f_.read(reinterpret_cast<char*>(v.data()), n * sizeof(T));
    }
    const std::string& path() const { return path_; }

private:
    std::string path_;
    std::ifstream f_;
};

class Out {
public:
    Out(const std::string& path, bool append) : f_(path, append ? std::ios::binary | std::ios::app : std::ios::binary) {}
    bool ok() const { return (bool)f_; }
    template <class T>
    void put(const T& v) { f_.write(reinterpret_cast<const char*>(&v), sizeof(T)); }
    template <class T>
    void put(const T* v, size_t n) { if (n) f_.write(reinterpret_cast<const char*>(v), n * sizeof(T)); }
    bool close()
    {
        f_.close();
        return !f_.fail();
    }

private:
    std::ofstream f_;
};

ug_status bad_file(const In& in) { return ferr(UG_EIO, "cannot read " + in.path() + " (missing or truncated)"); }

std::string join(const std::string& dir, const std::string& name)
{
    if (dir.empty() || dir.back() == '/') return dir + name;
    return dir + "/" + name;
}

// ---------------------------------------------------------------- libconfig subset
struct Cfg {
    std::map<std::string, std::map<std::string, std::string>> groups;
    bool num(const std::string& g, const std::string& k, double& v) const
    {
        auto gi = groups.find(g);
        if (gi == groups.end()) return false;
        auto ki = gi->second.find(k);
        if (ki == gi->second.end()) return false;
        v = std::strtod(ki->second.c_str(), nullptr);
        return true;
    }
};

ug_status parse_cfg(const std::string& path, Cfg& cfg)
{
    std::ifstream f(path);
    if (!f) return ferr(UG_EIO, "cannot read " + path);
    std::string t((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    // strip comments
    std::string s;
    for (size_t i = 0; i < t.size(); ++i) {
        if (t[i] == '"') {
            const size_t j = t.find('"', i + 1);
            const size_t e = j == std::string::npos ? t.size() : j + 1;
            s.append(t, i, e - i);
            i = e - 1;
        } else if (t.compare(i, 2, "/*") == 0) {
            const size_t j = t.find("*/", i + 2);
            i = j == std::string::npos ? t.size() : j + 1;
            s.push_back(' ');
        } else if (t.compare(i, 2, "//") == 0 || t[i] == '#') {
            while (i < t.size() && t[i] != '\n') ++i;
            s.push_back('\n');
        } else {
            s.push_back(t[i]);
        }
    }
    std::string group;
    size_t i = 0;
    auto skip = [&] { while (i < s.size() && std::isspace((unsigned char)s[i])) ++i; };
    while (true) {
        skip();
        if (i >= s.size()) break;
        if (s[i] == '}') {
            group.clear();
            ++i;
            skip();
            if (i < s.size() && (s[i] == ';' || s[i] == ',')) ++i;
            continue;
        }
        size_t j = i;
        while (j < s.size() && (std::isalnum((unsigned char)s[j]) || s[j] == '_')) ++j;
        if (j == i) return ferr(UG_EINVAL, path + ": unexpected character in a setting name");
        const std::string name = s.substr(i, j - i);
        i = j;
        skip();
        if (i >= s.size() || (s[i] != '=' && s[i] != ':')) return ferr(UG_EINVAL, path + ": expected '=' after " + name);
        ++i;
        skip();
        if (i < s.size() && s[i] == '{') {
            group = name;
            cfg.groups[group];
            ++i;
            continue;
        }
        size_t e = i;
        if (i < s.size() && s[i] == '"') {
            e = s.find('"', i + 1);
            if (e == std::string::npos) return ferr(UG_EINVAL, path + ": unterminated string");
            cfg.groups[group][name] = s.substr(i + 1, e - i - 1);
            i = e + 1;
        } else {
            while (e < s.size() && s[e] != ';' && s[e] != ',' && s[e] != '}' && s[e] != '\n') ++e;
            std::string v = s.substr(i, e - i);
            while (!v.empty() && std::isspace((unsigned char)v.back())) v.pop_back();
            cfg.groups[group][name] = v;
            i = e;
        }
        skip();
        if (i < s.size() && (s[i] == ';' || s[i] == ',')) ++i;
    }
    return UG_OK;
}

std::string ending(int trial) { return trial > 0 ? "_" + std::to_string(trial) : std::string(); }

// per-source lists of a CSR: (id, count, then id int + 3 doubles per target)
ug_status read_connections(const std::string& path, int n_expect, std::vector<int32_t>& off, std::vector<int32_t>& tgt,
                           std::vector<double>& w, std::vector<double>& len, std::vector<double>& d)
{
    In in(path);
    int32_t n = 0;
    if (!in.ok() || !in.get(n)) return bad_file(in);
    if (n != n_expect) return ferr(UG_EINVAL, path + ": neuron count differs from num_neurons.bin");
    off.assign(1, 0);
    tgt.clear(); w.clear(); len.clear(); d.clear();
    for (int i = 0; i < n; ++i) {
        int32_t id = 0, k = 0;
        if (!in.get(id) || !in.get(k) || k < 0) return bad_file(in);
        for (int j = 0; j < k; ++j) {
            int32_t t;
            double a, b, c;
            if (!in.get(t) || !in.get(a) || !in.get(b) || !in.get(c)) return bad_file(in);
            tgt.push_back(t); w.push_back(a); len.push_back(b); d.push_back(c);
        }
        off.push_back((int32_t)tgt.size());
    }
    return UG_OK;
}

ug_status read_lists(const std::string& path, int n_expect, std::vector<int32_t>& off, std::vector<int32_t>& tgt)
{
    In in(path);
    int32_t n = 0, trial = 0;
    if (!in.ok() || !in.get(n) || !in.get(trial)) return bad_file(in);
    if (n != n_expect) return ferr(UG_EINVAL, path + ": neuron count differs from num_neurons.bin");
    off.assign(1, 0);
    tgt.clear();
    for (int i = 0; i < n; ++i) {
        int32_t k = 0;
        std::vector<int32_t> row;
        if (!in.get(k) || k < 0 || !in.get(row, (size_t)k)) return bad_file(in);
        tgt.insert(tgt.end(), row.begin(), row.end());
        off.push_back((int32_t)tgt.size());
    }
    return UG_OK;
}

ug_status read_ints(const std::string& path, int n_expect, std::vector<int32_t>& v)
{
    In in(path);
    int32_t n = 0, trial = 0;
    if (!in.ok() || !in.get(n) || !in.get(trial) || n != n_expect || !in.get(v, (size_t)n)) return bad_file(in);
    return UG_OK;
}

ug_status read_delays(const std::string& path, int n_expect, std::vector<std::vector<double>>& rows)
{
    In in(path);
    int32_t n = 0, trial = 0;
    if (!in.ok() || !in.get(n) || !in.get(trial) || n != n_expect) return bad_file(in);
    rows.assign(n, {});
    for (int i = 0; i < n; ++i) {
        int32_t k = 0;
        if (!in.get(k) || k < 0 || !in.get(rows[i], (size_t)k)) return bad_file(in);
    }
    return UG_OK;
}

ug_status read_coords(const std::string& path, int n_expect, std::vector<double>& xyz, double& model)
{
    In in(path);
    int32_t n = 0, dim = 0;
    if (!in.ok() || !in.get(n) || !in.get(dim) || !in.get(model) || n != n_expect) return bad_file(in);
    std::vector<double> raw;
    if (dim < 1 || dim > 3 || !in.get(raw, (size_t)n * dim)) return bad_file(in);
    xyz.assign((size_t)3 * n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int c = 0; c < dim; ++c) xyz[(size_t)3 * i + c] = raw[(size_t)dim * i + c];
    return UG_OK;
}

// ---------------------------------------------------------------- writers
void write_connections(Out& o, int n, const std::vector<int32_t>& off, const std::vector<int32_t>& tgt,
                       const std::vector<double>& w, const std::vector<double>& len, const std::vector<double>& d)
{
    o.put((int32_t)n);
    for (int32_t i = 0; i < n; ++i) {
        o.put(i);
        o.put((int32_t)(off[i + 1] - off[i]));
        for (int32_t k = off[i]; k < off[i + 1]; ++k) {
            o.put(tgt[k]); o.put(w[k]); o.put(len[k]); o.put(d[k]);
        }
    }
}

// write_coordinates (:18431-18500): 3 coordinates per neuron on the sphere, x and y on the square
void write_coords(Out& o, int n, const std::vector<double>& xyz, double model, int dim = 3)
{
    o.put((int32_t)n);
    o.put((int32_t)dim);
    o.put(model);
    if (dim == 3) {
        o.put(xyz.data(), xyz.size());
        return;
    }
    for (int i = 0; i < n; ++i) o.put(&xyz[3 * (size_t)i], (size_t)dim);
}

ug_status closed(Out& o, const std::string& path)
{
    return o.close() ? UG_OK : ferr(UG_EIO, "cannot write " + path);
}

struct Conn {
    std::vector<int32_t> off, tgt;
    std::vector<double> w, d, len;
};

ug_status get_conn(ug_ctx* ctx, int32_t net, int which, int nsrc, Conn& c)
{
    int64_t total = 0;
    UG_FTRY(ug_get_connections(ctx, net, which, nullptr, nullptr, nullptr, nullptr, &total));
    c.off.resize(nsrc + 1);
    c.tgt.resize(total); c.w.resize(total); c.d.resize(total); c.len.resize(total);
    UG_FTRY(ug_get_connections(ctx, net, which, c.off.data(), c.tgt.data(), c.w.data(), c.d.data(), &total));
    return ug_get_connection_lengths(ctx, net, which, c.len.data());
}

ug_status get_lists(ug_ctx* ctx, int32_t net, int which, int n, std::vector<int32_t>& off, std::vector<int32_t>& tgt)
{
    int64_t total = 0;
    UG_FTRY(ug_get_synapse_list(ctx, net, which, nullptr, nullptr, &total));
    off.resize(n + 1);
    tgt.resize(total);
    return ug_get_synapse_list(ctx, net, which, off.data(), tgt.data(), &total);
}

ug_status write_spikes(ug_ctx* ctx, int32_t net, int which, int n, int32_t trial, const std::string& path,
                       int instance = 0)
{
    int64_t cnt = 0;
    std::vector<int32_t> nid, step;
    if (ug_get_spikes(ctx, net, instance, which, nullptr, nullptr, 0, &cnt) == UG_OK) {
        nid.resize(cnt); step.resize(cnt);
        UG_FTRY(ug_get_spikes(ctx, net, instance, which, nid.data(), step.data(), cnt, &cnt));
    }   // a network that has run no trial writes empty lists
    std::vector<std::vector<double>> t(n);
    for (int64_t k = 0; k < cnt; ++k) {
        double x = 0.0;
        UG_FTRY(ug_step_time(ctx, net, step[k], &x));
        t[nid[k]].push_back(x);
    }
    Out o(path, false);
    if (!o.ok()) return ferr(UG_EIO, "cannot write " + path);
    const double duration = 500.0;   // TRIAL_DURATION (NetworkGrowthSimulator.cpp:17)
    o.put(trial);
    o.put(duration);
    o.put((int32_t)n);
    for (int i = 0; i < n; ++i) {
        o.put((int32_t)t[i].size());
        o.put(t[i].data(), t[i].size());
    }
    return closed(o, path);
}

}  // namespace

extern "C" {

ug_status ug_load_network_dir(ug_ctx* ctx, const char* dir_c, int32_t starting_trial, int32_t num_steps,
                              uint64_t seed, int32_t stream_id, int32_t* net_id)
{
    if (!ctx || !dir_c || !net_id) return ferr(UG_EINVAL, "null argument");
    const std::string dir(dir_c), e = ending(starting_trial);
    ug_network_desc d;
    std::memset(&d, 0, sizeof(d));
    // configuration files: growth and topology parameters
    Cfg g, t;
    UG_FTRY(parse_cfg(join(dir, "growth_parameters.cfg"), g));
    UG_FTRY(parse_cfg(join(dir, "network_parameters.cfg"), t));
    auto num = [](const Cfg& c, const char* grp, const char* key, double dflt) {
        double v = dflt;
        c.num(grp, key, v);
        return v;
    };
    d.syn.Nss = (int32_t)num(g, "synapticParameters", "Nss", 0);
    const char* sp = "synapticParameters";
    d.syn.A_P = num(g, sp, "A_P", 0); d.syn.A_D = num(g, sp, "A_D", 0); d.syn.T_0 = num(g, sp, "T_0", 0);
    d.syn.T_P = num(g, sp, "T_P", 0); d.syn.T_D = num(g, sp, "T_D", 0); d.syn.TAU_P = num(g, sp, "TAU_P", 0);
    d.syn.TAU_D = num(g, sp, "TAU_D", 0); d.syn.BETA = num(g, sp, "BETA", 0);
    d.syn.BETA_SUPERSYNAPSE = num(g, sp, "BETA_SUPERSYNAPSE", 0);
    d.syn.ACTIVATION_THRESHOLD = num(g, sp, "ACTIVATION_THRESHOLD", 0);
    d.syn.SUPERSYNAPSE_THRESHOLD = num(g, sp, "SUPERSYNAPSE_THRESHOLD", 0);
    d.syn.WEIGHT_MAX = num(g, sp, "WEIGHT_MAX", 0);
    const char* mp = "maturationParameters";
    d.mat.E_REST_MATURE = num(g, mp, "E_REST_MATURE", 0); d.mat.E_REST_IMMATURE = num(g, mp, "E_REST_IMMATURE", 0);
    d.mat.GCA_MATURE = num(g, mp, "GCA_MATURE", 0); d.mat.GCA_IMMATURE = num(g, mp, "GCA_IMMATURE", 0);
    d.mat.DEATH_RATE_THRESHOLD = num(g, mp, "DEATH_RATE_THRESHOLD", 0);
    d.mat.RATE_WINDOW_LONG = (int32_t)num(g, mp, "RATE_WINDOW_LONG", 0);
    const char* np = "noiseParameters";
    d.noise.white_noise_mean_soma = num(g, np, "white_noise_mean_soma", 0);
    d.noise.white_noise_std_soma = num(g, np, "white_noise_std_soma", 0);
    d.noise.white_noise_mean_dend = num(g, np, "white_noise_mean_dend", 0);
    d.noise.white_noise_std_dend = num(g, np, "white_noise_std_dend", 0);
    const char* cp = "connectionParameters";
    d.conn.Gei_max = num(g, cp, "Gei_max", 0); d.conn.Gie_max = num(g, cp, "Gie_max", 0);
    d.conn.delay_constant = num(g, cp, "delay_constant", 0);
    const char* tp = "spatialParameters";
    d.conn.A_RA2I = num(t, tp, "A_RA2I", 0); d.conn.SIGMA_RA2I = num(t, tp, "SIGMA_RA2I", 0);
    d.conn.B_I2RA = num(t, tp, "B_I2RA", 0); d.conn.SIGMA_I2RA = num(t, tp, "SIGMA_I2RA", 0);
    // sizes and training (read_number_of_neurons, read_training_neurons / _spread)
    int32_t nra = 0, ni = 0;
    {
        In in(join(dir, "num_neurons.bin"));
        if (!in.ok() || !in.get(nra) || !in.get(ni) || nra <= 0 || ni < 0) return bad_file(in);
    }
    std::vector<int32_t> training;
    std::vector<double> spread;
    {
        In a(join(dir, "training_neurons.bin")), b(join(dir, "training_spread.bin"));
        int32_t k = 0, k2 = 0;
        if (!a.ok() || !a.get(k) || k < 0 || !a.get(training, (size_t)k)) return bad_file(a);
        if (!b.ok() || !b.get(k2) || k2 != k || !b.get(spread, (size_t)k2)) return bad_file(b);
        // the reference sorts the neurons after reading, and pairs the k-th sorted
        // neuron with the k-th spread time of the file (:1998-1999, :5669)
        std::sort(training.begin(), training.end());
    }
    std::vector<double> ra_xyz, i_xyz, model_i = {0.0};
    double model = 0.0;
    UG_FTRY(read_coords(join(dir, "RA_xy" + e + ".bin"), nra, ra_xyz, model));
    UG_FTRY(read_coords(join(dir, "I_xy.bin"), ni, i_xyz, model_i[0]));
    d.conn.model_interneuron_distance = model;   // read_all_coordinates takes it from RA_xy
    Conn ri, ir;
    UG_FTRY(read_connections(join(dir, "RA_I_connections" + e + ".bin"), nra, ri.off, ri.tgt, ri.w, ri.len, ri.d));
    UG_FTRY(read_connections(join(dir, "I_RA_connections" + e + ".bin"), ni, ir.off, ir.tgt, ir.w, ir.len, ir.d));
    std::vector<int32_t> act_off, act_tgt, sup_off, sup_tgt;
    UG_FTRY(read_lists(join(dir, "RA_RA_super_connections" + e + ".bin"), nra, sup_off, sup_tgt));
    UG_FTRY(read_lists(join(dir, "RA_RA_active_connections" + e + ".bin"), nra, act_off, act_tgt));
    std::vector<double> W;
    {
        In in(join(dir, "weights" + e + ".bin"));
        int32_t n = 0, trial = 0;
        if (!in.ok() || !in.get(n) || !in.get(trial) || n != nra || !in.get(W, (size_t)nra * nra)) return bad_file(in);
    }
    std::vector<std::vector<double>> drr, dri, dir_;
    UG_FTRY(read_delays(join(dir, "axonal_delays_RA2RA" + e + ".bin"), nra, drr));
    UG_FTRY(read_delays(join(dir, "axonal_delays_RA2I" + e + ".bin"), nra, dri));
    UG_FTRY(read_delays(join(dir, "axonal_delays_I2RA" + e + ".bin"), ni, dir_));
    std::vector<double> D((size_t)nra * nra, 0.0);
    for (int i = 0; i < nra; ++i) {
        if ((int)drr[i].size() != nra) return ferr(UG_EINVAL, "axonal_delays_RA2RA: a row is not dense");
        std::copy(drr[i].begin(), drr[i].end(), D.begin() + (size_t)i * nra);
        if ((int)dri[i].size() != ri.off[i + 1] - ri.off[i]) return ferr(UG_EINVAL, "axonal_delays_RA2I: row sizes");
        std::copy(dri[i].begin(), dri[i].end(), ri.d.begin() + ri.off[i]);
    }
    for (int i = 0; i < ni; ++i) {
        if ((int)dir_[i].size() != ir.off[i + 1] - ir.off[i]) return ferr(UG_EINVAL, "axonal_delays_I2RA: row sizes");
        std::copy(dir_[i].begin(), dir_[i].end(), ir.d.begin() + ir.off[i]);
    }
    // neuron state (read_activity_history, read_replacement_history, read_remodeled_indicators,
    // read_maturation_properties)
    const int win = d.mat.RATE_WINDOW_LONG;
    std::vector<int32_t> hist;
    {
        In in(join(dir, "activity_history" + e + ".bin"));
        int32_t n = 0, w = 0, trial = 0;
        if (!in.ok() || !in.get(n) || !in.get(w) || !in.get(trial) || n != nra || w != win ||
            !in.get(hist, (size_t)nra * win))
            return bad_file(in);
    }
    std::vector<int32_t> tar, remod, mature(nra), scale_i(nra);
    UG_FTRY(read_ints(join(dir, "replacement_history" + e + ".bin"), nra, tar));
    UG_FTRY(read_ints(join(dir, "remodeled_indicators" + e + ".bin"), nra, remod));
    std::vector<double> rest(nra), gca(nra), scale(nra);
    {
        In in(join(dir, "maturation_properties" + e + ".bin"));
        int32_t n = 0, trial = 0;
        if (!in.ok() || !in.get(n) || !in.get(trial) || n != nra) return bad_file(in);
        for (int i = 0; i < nra; ++i)
            if (!in.get(mature[i]) || !in.get(scale_i[i]) || !in.get(rest[i]) || !in.get(gca[i])) return bad_file(in);
        for (int i = 0; i < nra; ++i) scale[i] = (double)scale_i[i];
    }
    d.n_ra = nra;
    d.n_i = ni;
    d.num_steps = num_steps > 0 ? num_steps : 25000;
    d.net_id = stream_id;
    d.seed = seed;
    d.ra2i_off = ri.off.data(); d.ra2i_tgt = ri.tgt.data(); d.ra2i_w = ri.w.data(); d.ra2i_d = ri.d.data();
    d.ra2i_len = ri.len.data();
    d.i2ra_off = ir.off.data(); d.i2ra_tgt = ir.tgt.data(); d.i2ra_w = ir.w.data(); d.i2ra_d = ir.d.data();
    d.i2ra_len = ir.len.data();
    d.w_rara = W.data(); d.d_rara = D.data();
    std::vector<double> L((size_t)nra * nra, 0.0);   // RA->RA lengths are not in the state files:
    if (d.conn.delay_constant != 0.0)                // delays are length * 0.01 * delay_constant
        for (size_t k = 0; k < L.size(); ++k) L[k] = D[k] / (0.01 * d.conn.delay_constant);
    d.len_rara = L.data();
    d.active_off = act_off.data(); d.active_tgt = act_tgt.data();
    d.super_off = sup_off.data(); d.super_tgt = sup_tgt.data();
    d.rest_potential = rest.data(); d.gca = gca.data();
    d.mature = mature.data(); d.maturation_scale = scale.data();
    d.remodeled = remod.data(); d.trials_after_replacement = tar.data();
    d.activity_history = hist.data();
    d.n_tr = (int32_t)training.size();
    d.training = training.data(); d.training_spread = spread.data();
    d.ra_xyz = ra_xyz.data(); d.i_xyz = i_xyz.data();
    return ug_load_network(ctx, &d, net_id);
}

ug_status ug_write_state_dir(ug_ctx* ctx, int32_t net, const char* dir_c, const char* file_ending,
                             int32_t trial_number)
{
    if (!ctx || !dir_c) return ferr(UG_EINVAL, "null argument");
    const std::string dir(dir_c), e(file_ending ? file_ending : "");
    ug_network_info info;
    UG_FTRY(ug_get_network_info(ctx, net, &info));
    const int n = info.n_ra, ni = info.n_i;
    const int32_t trial = trial_number;
    std::vector<double> W((size_t)n * n), D((size_t)n * n);
    UG_FTRY(ug_get_weights(ctx, net, W.data()));
    UG_FTRY(ug_get_delays(ctx, net, D.data()));
    Conn ri, ir;
    UG_FTRY(get_conn(ctx, net, 0, n, ri));
    UG_FTRY(get_conn(ctx, net, 1, ni, ir));
    std::vector<double> ra_xyz((size_t)3 * n), i_xyz((size_t)3 * ni);
    UG_FTRY(ug_get_coordinates(ctx, net, ra_xyz.data(), i_xyz.data()));
    // write_alterable_network: RA_xy, RA_I / I_RA connections
    {
        const std::string p = join(dir, "RA_xy" + e + ".bin");
        Out o(p, false);
        write_coords(o, n, ra_xyz, info.conn.model_interneuron_distance);
        UG_FTRY(closed(o, p));
        const std::string p1 = join(dir, "RA_I_connections" + e + ".bin"), p2 = join(dir, "I_RA_connections" + e + ".bin");
        Out a(p1, false), b(p2, false);
        write_connections(a, n, ri.off, ri.tgt, ri.w, ri.len, ri.d);
        write_connections(b, ni, ir.off, ir.tgt, ir.w, ir.len, ir.d);
        UG_FTRY(closed(a, p1));
        UG_FTRY(closed(b, p2));
    }
    // write_weights
    {
        const std::string p = join(dir, "weights" + e + ".bin");
        Out o(p, false);
        o.put((int32_t)n); o.put(trial);
        o.put(W.data(), W.size());
        UG_FTRY(closed(o, p));
    }
    // write_weight_statistics: row sums accumulated row by row, then the deviations in one sum
    {
        const std::string p = join(dir, "weight_statistics.bin");
        Out o(p, trial != 0);
        double mean = 0.0;
        for (int i = 0; i < n; ++i) mean += std::accumulate(W.begin() + (size_t)i * n, W.begin() + (size_t)(i + 1) * n, 0.0);
        mean /= ((double)n * (double)n);
        double sd = 0.0;
        for (double w : W) sd += (w - mean) * (w - mean);
        if ((long long)n * n > 1) sd = std::sqrt(sd / ((double)n * (double)n - 1));
        o.put(trial); o.put(mean); o.put(sd);
        UG_FTRY(closed(o, p));
    }
    // write_axonal_delays x 3
    {
        const std::string p = join(dir, "axonal_delays_RA2RA" + e + ".bin");
        Out o(p, false);
        o.put((int32_t)n); o.put(trial);
        for (int i = 0; i < n; ++i) {
            o.put((int32_t)n);
            o.put(D.data() + (size_t)i * n, (size_t)n);
        }
        UG_FTRY(closed(o, p));
        for (int which = 0; which < 2; ++which) {
            const Conn& c = which == 0 ? ri : ir;
            const int nsrc = which == 0 ? n : ni;
            const std::string q = join(dir, std::string(which == 0 ? "axonal_delays_RA2I" : "axonal_delays_I2RA") + e + ".bin");
            Out oq(q, false);
            oq.put((int32_t)nsrc); oq.put(trial);
            for (int i = 0; i < nsrc; ++i) {
                oq.put((int32_t)(c.off[i + 1] - c.off[i]));
                oq.put(c.d.data() + c.off[i], (size_t)(c.off[i + 1] - c.off[i]));
            }
            UG_FTRY(closed(oq, q));
        }
    }
    // write_super_synapses / write_active_synapses
    for (int which = 1; which >= 0; --which) {
        std::vector<int32_t> off, tgt;
        UG_FTRY(get_lists(ctx, net, which, n, off, tgt));
        const std::string p = join(dir, std::string(which ? "RA_RA_super_connections" : "RA_RA_active_connections") + e + ".bin");
        Out o(p, false);
        o.put((int32_t)n); o.put(trial);
        for (int i = 0; i < n; ++i) {
            o.put((int32_t)(off[i + 1] - off[i]));
            o.put(tgt.data() + off[i], (size_t)(off[i + 1] - off[i]));
        }
        UG_FTRY(closed(o, p));
    }
    // neuron properties
    std::vector<double> rest(n), gca(n), scale(n), frl(n);
    std::vector<int32_t> mature(n), remod(n), tar(n);
    UG_FTRY(ug_get_neuron_props(ctx, net, rest.data(), gca.data(), mature.data(), scale.data(), remod.data(),
                                tar.data(), frl.data()));
    auto ints = [&](const char* name, const std::vector<int32_t>& v) -> ug_status {
        const std::string p = join(dir, std::string(name) + e + ".bin");
        Out o(p, false);
        o.put((int32_t)n); o.put(trial);
        o.put(v.data(), v.size());
        return closed(o, p);
    };
    UG_FTRY(ints("mature", mature));
    {
        const std::string p = join(dir, "maturation_properties" + e + ".bin");
        Out o(p, false);
        o.put((int32_t)n); o.put(trial);
        for (int i = 0; i < n; ++i) {
            o.put(mature[i]);
            o.put((int32_t)scale[i]);   // maturation_scale_global is int in the reference
            o.put(rest[i]);
            o.put(gca[i]);
        }
        UG_FTRY(closed(o, p));
    }
    {
        const int win = info.mat.RATE_WINDOW_LONG;
        std::vector<int32_t> hist((size_t)n * std::max(win, 0));
        if (win > 0) UG_FTRY(ug_get_activity_history(ctx, net, hist.data()));
        const std::string p = join(dir, "activity_history" + e + ".bin");
        Out o(p, false);
        o.put((int32_t)n); o.put((int32_t)win); o.put(trial);
        o.put(hist.data(), hist.size());
        UG_FTRY(closed(o, p));
    }
    UG_FTRY(ints("replacement_history", tar));
    UG_FTRY(ints("remodeled_indicators", remod));
    // spike times of the last trial
    UG_FTRY(write_spikes(ctx, net, 0, n, trial, join(dir, "spike_times_soma" + e + ".bin")));
    UG_FTRY(write_spikes(ctx, net, 1, n, trial, join(dir, "spike_times_dend" + e + ".bin")));
    UG_FTRY(write_spikes(ctx, net, 2, ni, trial, join(dir, "spike_times_interneuron" + e + ".bin")));
    return UG_OK;
}

ug_status ug_write_topology_dir(ug_ctx* ctx, int32_t net, const char* dir_c)
{
    if (!ctx || !dir_c) return ferr(UG_EINVAL, "null argument");
    const std::string dir(dir_c);
    ug_network_info info;
    UG_FTRY(ug_get_network_info(ctx, net, &info));
    const int n = info.n_ra, ni = info.n_i;
    std::vector<double> ra_xyz((size_t)3 * n), i_xyz((size_t)3 * ni);
    UG_FTRY(ug_get_coordinates(ctx, net, ra_xyz.data(), i_xyz.data()));
    Conn ri, ir;
    UG_FTRY(get_conn(ctx, net, 0, n, ri));
    UG_FTRY(get_conn(ctx, net, 1, ni, ir));
    const double model = info.conn.model_interneuron_distance;
    struct F { const char* name; int k; } files[] = {{"I_xy.bin", 0}, {"RA_xy.bin", 1}};
    for (const F& f : files) {
        const std::string p = join(dir, f.name);
        Out o(p, false);
        write_coords(o, f.k ? n : ni, f.k ? ra_xyz : i_xyz, model);
        UG_FTRY(closed(o, p));
    }
    const std::string p1 = join(dir, "RA_I_connections.bin"), p2 = join(dir, "I_RA_connections.bin");
    Out a(p1, false), b(p2, false);
    write_connections(a, n, ri.off, ri.tgt, ri.w, ri.len, ri.d);
    write_connections(b, ni, ir.off, ir.tgt, ir.w, ir.len, ir.d);
    UG_FTRY(closed(a, p1));
    UG_FTRY(closed(b, p2));
    {
        const std::string p = join(dir, "num_neurons.bin");
        Out o(p, false);
        o.put((int32_t)n); o.put((int32_t)ni);
        UG_FTRY(closed(o, p));
    }
    // training files, neurons ascending (the order the reference reads them back in)
    std::vector<int32_t> tr(info.n_tr);
    std::vector<double> sp(info.n_tr);
    UG_FTRY(ug_get_training(ctx, net, tr.data(), sp.data()));
    std::vector<int> order(info.n_tr);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int x, int y) { return tr[x] < tr[y]; });
    const std::string pn = join(dir, "training_neurons.bin"), ps = join(dir, "training_spread.bin");
    Out on(pn, false), os(ps, false);
    on.put((int32_t)info.n_tr);
    os.put((int32_t)info.n_tr);
    for (int k : order) {
        on.put(tr[k]);
        os.put(sp[k]);
    }
    UG_FTRY(closed(on, pn));
    return closed(os, ps);
}

ug_status ug_append_num_synapses(ug_ctx* ctx, int32_t net, const char* path, int32_t trial)
{
    if (!ctx || !path) return ferr(UG_EINVAL, "null argument");
    int64_t act = 0, sup = 0;
    UG_FTRY(ug_get_synapse_list(ctx, net, 0, nullptr, nullptr, &act));
    UG_FTRY(ug_get_synapse_list(ctx, net, 1, nullptr, nullptr, &sup));
    Out o(path, trial != 0);
    o.put(trial); o.put((int32_t)act); o.put((int32_t)sup);
    return closed(o, path);
}

ug_status ug_append_replaced(ug_ctx* ctx, int32_t net, const char* path, int32_t trial)
{
    if (!ctx || !path) return ferr(UG_EINVAL, "null argument");
    int64_t k = 0;
    UG_FTRY(ug_get_replaced(ctx, net, nullptr, 0, &k));
    std::vector<int32_t> ids(k);
    UG_FTRY(ug_get_replaced(ctx, net, ids.data(), k, &k));
    Out o(path, trial != 0);
    o.put(trial); o.put((int32_t)k);
    o.put(ids.data(), ids.size());
    return closed(o, path);
}

ug_status ug_write_jitter(ug_ctx* ctx, int32_t net, const char* path)
{
    if (!ctx || !path) return ferr(UG_EINVAL, "null argument");
    ug_network_info info;
    UG_FTRY(ug_get_network_info(ctx, net, &info));
    const int n = info.n_ra;
    const int B = info.batch;
    if (B == 0) return ferr(UG_EINVAL, "no test batch has run on this network");
    std::vector<int32_t> cs((size_t)B * n), fs((size_t)B * n), cd((size_t)B * n), fd((size_t)B * n);
    UG_FTRY(ug_get_trial_stats(ctx, net, 0, cs.data(), fs.data()));
    UG_FTRY(ug_get_trial_stats(ctx, net, 1, cd.data(), fd.data()));
    Out o(path, false);
    o.put((int32_t)n); o.put((int32_t)B);
    for (int i = 0; i < n; ++i) {
        for (int which = 0; which < 2; ++which) {
            const std::vector<int32_t>& c = which ? cd : cs;
            const std::vector<int32_t>& f = which ? fd : fs;
            std::vector<double> first;
            double spikes = 0.0;
            for (int b = 0; b < B; ++b) {
                spikes += c[(size_t)b * n + i];
                if (f[(size_t)b * n + i] >= 0) {
                    double t = 0.0;
                    UG_FTRY(ug_step_time(ctx, net, f[(size_t)b * n + i], &t));
                    first.push_back(t);
                }
            }
            const double k = (double)first.size();
            const double mean = first.empty() ? -1.0 : std::accumulate(first.begin(), first.end(), 0.0) / k;
            double acc = 0.0;
            for (double t : first) acc += (t - mean) * (t - mean);
            const double sd = first.size() > 1 ? std::sqrt(acc / (k - 1)) : -1.0;
            const double prob = k / (double)B, avg = spikes / (double)B;
            o.put(prob); o.put(avg); o.put(mean); o.put(sd);
        }
    }
    return closed(o, path);
}

// set_recording's files (NetworkGrowthSimulator.cpp:2352-2407): per recorded neuron,
// RA/RA<id>_trial<t>.bin or I/I<id>_trial<t>.bin of (time, state) records of doubles, in
// whole buffers of 1000 records as write_buffers appends them (HH2_test.cpp:394-411,
// HHI_buffer.cpp:720-734); the trial's last partial buffer is never written.
ug_status ug_write_traces(ug_ctx* ctx, int32_t net, const char* dir, int32_t trial_number)
{
    if (!ctx || !dir) return ferr(UG_EINVAL, "null argument");
    int32_t nra = 0, ni = 0;
    UG_FTRY(ug_get_recording(ctx, net, nullptr, &nra, nullptr, &ni));
    std::vector<int32_t> ra((size_t)std::max(nra, 1)), in((size_t)std::max(ni, 1));
    UG_FTRY(ug_get_recording(ctx, net, ra.data(), &nra, in.data(), &ni));
    const int kBuffer = 1000;   // HH2_test::BUFFER_SIZE, HHI_buffer's likewise
    for (int which = 0; which < 2; ++which) {
        const int cnt = which == 0 ? nra : ni;
        if (cnt == 0) continue;
        const std::string sub = join(dir, which == 0 ? "RA" : "I");
        if (::mkdir(sub.c_str(), 0755) != 0 && errno != EEXIST) return ferr(UG_EIO, "cannot create " + sub);
        for (int k = 0; k < cnt; ++k) {
            int32_t records = 0;
            UG_FTRY(ug_get_trace(ctx, net, which, k, nullptr, &records));
            const int w = which == 0 ? 5 : 4;
            std::vector<double> rec((size_t)records * w);
            UG_FTRY(ug_get_trace(ctx, net, which, k, rec.data(), &records));
            const int id = which == 0 ? ra[k] : in[k];
            const std::string path = join(sub, std::string(which == 0 ? "RA" : "I") + std::to_string(id) + "_trial" +
                                                   std::to_string(trial_number) + ".bin");
            Out o(path, false);
            const size_t whole = (size_t)(records / kBuffer) * kBuffer;
            for (size_t r = 0; r < whole; ++r)
                for (int c = 0; c < w; ++c) o.put(rec[r * w + c]);
            UG_FTRY(closed(o, path));
        }
    }
    return UG_OK;
}

ug_status ug_write_spike_times(ug_ctx* ctx, int32_t net, int32_t instance, int32_t which, const char* path,
                               int32_t trial_number)
{
    if (!ctx || !path) return ferr(UG_EINVAL, "null argument");
    if (which < 0 || which > 2) return ferr(UG_EINVAL, "which must be 0, 1 or 2");
    ug_network_info info;
    UG_FTRY(ug_get_network_info(ctx, net, &info));
    if (instance < 0 || instance >= info.batch) return ferr(UG_EINVAL, "instance out of range");
    return write_spikes(ctx, net, which, which == 2 ? info.n_i : info.n_ra, trial_number, path, instance);
}

ug_status ug_write_graph_state(ug_ctx* ctx, int32_t net, const char* dir_c, int32_t trial_number)
{
    if (!ctx || !dir_c) return ferr(UG_EINVAL, "null argument");
    const std::string dir(dir_c);
    ug_network_info info;
    UG_FTRY(ug_get_network_info(ctx, net, &info));
    const int n = info.n_ra;
    UG_FTRY(ug_append_num_synapses(ctx, net, join(dir, "num_synapses.bin").c_str(), trial_number));
    UG_FTRY(write_spikes(ctx, net, 0, n, trial_number, join(dir, "spike_times_soma.bin")));
    UG_FTRY(write_spikes(ctx, net, 1, n, trial_number, join(dir, "spike_times_dend.bin")));
    UG_FTRY(write_spikes(ctx, net, 2, info.n_i, trial_number, join(dir, "spike_times_interneuron.bin")));
    for (int which = 1; which >= 0; --which) {
        std::vector<int32_t> off, tgt;
        UG_FTRY(get_lists(ctx, net, which, n, off, tgt));
        const std::string p = join(dir, which ? "RA_RA_super_connections.bin" : "RA_RA_active_connections.bin");
        Out o(p, false);
        o.put((int32_t)n); o.put(trial_number);
        for (int i = 0; i < n; ++i) {
            o.put((int32_t)(off[i + 1] - off[i]));
            o.put(tgt.data() + off[i], (size_t)(off[i + 1] - off[i]));
        }
        UG_FTRY(closed(o, p));
    }
    return UG_OK;
}

// write_inhibition_tracking_state (:18606-18618)
ug_status ug_write_inhibition_tracking_state(ug_ctx* ctx, int32_t net, const char* dir_c, int32_t trial_number)
{
    if (!ctx || !dir_c) return ferr(UG_EINVAL, "null argument");
    const std::string dir(dir_c), e = "_" + std::to_string(trial_number);
    ug_network_info info;
    UG_FTRY(ug_get_network_info(ctx, net, &info));
    const int n = info.n_ra;
    int32_t points = 0;
    double res = 0.0;
    UG_FTRY(ug_get_inhibitory_conductance(ctx, net, nullptr, &points, &res));
    std::vector<double> g((size_t)n * points);
    UG_FTRY(ug_get_inhibitory_conductance(ctx, net, g.data(), &points, &res));
    // write_num_synapses: a new file at trial 0, appended to afterwards (:17885-17912)
    UG_FTRY(ug_append_num_synapses(ctx, net, join(dir, "num_synapses" + e + ".bin").c_str(), trial_number));
    UG_FTRY(write_spikes(ctx, net, 0, n, trial_number, join(dir, "spike_times_soma" + e + ".bin")));
    UG_FTRY(write_spikes(ctx, net, 1, n, trial_number, join(dir, "spike_times_dend" + e + ".bin")));
    UG_FTRY(write_spikes(ctx, net, 2, info.n_i, trial_number, join(dir, "spike_times_interneuron" + e + ".bin")));
    // write_inhibitory_conductance (:17689-17709)
    const std::string p = join(dir, "Ginh_trial" + e + ".bin");
    Out o(p, false);
    o.put((int32_t)n);
    o.put(points);
    o.put(res);
    o.put(g.data(), g.size());
    return closed(o, p);
}

}  // extern "C"

namespace {

const char* const kSynFields[] = {"A_P", "A_D", "T_0", "T_P", "T_D", "TAU_P", "TAU_D", "BETA", "BETA_SUPERSYNAPSE",
                                  "ACTIVATION_THRESHOLD", "SUPERSYNAPSE_THRESHOLD", "WEIGHT_MAX"};
const char* const kMatFields[] = {"E_GABA_MATURE", "E_GABA_IMMATURE", "E_REST_MATURE", "E_REST_IMMATURE",
                                  "AD_MATURE", "AD_IMMATURE", "GK_MATURE", "GK_IMMATURE", "GNA_MATURE",
                                  "GNA_IMMATURE", "GCA_MATURE", "GCA_IMMATURE", "GCAK_MATURE", "GCAK_IMMATURE",
                                  "GSL_MATURE", "GSL_IMMATURE", "GDL_MATURE", "GDL_IMMATURE", "RC_MATURE",
                                  "RC_IMMATURE"};

std::string fixed6(double v)
{
    char b[64];
    std::snprintf(b, sizeof(b), "%.6f", v);
    return b;
}

// ConfigurationNetworkGrowth::write_configuration (ConfigurationNetworkGrowth.cpp:210-295):
// std::fixed with six decimals from A_P on, blank lines as it places them.
ug_status write_growth_cfg(const std::string& path, const Cfg& c)
{
    auto v = [&](const char* g, const char* k) {
        double x = 0.0;
        c.num(g, k, x);
        return x;
    };
    std::string o = "synapticParameters = \n{\n\tNss = " + std::to_string((long)v("synapticParameters", "Nss")) + ";\n\n";
    for (const char* k : kSynFields) {
        o += std::string("\t") + k + " = " + fixed6(v("synapticParameters", k)) + ";\n";
        if (!std::strcmp(k, "TAU_D") || !std::strcmp(k, "BETA_SUPERSYNAPSE") || !std::strcmp(k, "WEIGHT_MAX")) o += "\n";
    }
    o += "};\n\nmaturationParameters = \n{\n";
    for (const char* k : kMatFields) {
        o += std::string("\t") + k + " = " + fixed6(v("maturationParameters", k)) + ";\n";
        if (std::strstr(k, "_IMMATURE")) o += "\n";
    }
    o += "\tDEATH_RATE_THRESHOLD = " + fixed6(v("maturationParameters", "DEATH_RATE_THRESHOLD")) + ";\n\n";
    o += "\tRATE_WINDOW_LONG = " + std::to_string((long)v("maturationParameters", "RATE_WINDOW_LONG")) + ";\n\n";
    o += "};\n\nnoiseParameters = \n{\n";
    for (const char* k : {"white_noise_mean_soma", "white_noise_std_soma", "white_noise_mean_dend", "white_noise_std_dend"})
        o += std::string("\t") + k + " = " + fixed6(v("noiseParameters", k)) + ";\n";
    o += "};\n\nconnectionParameters = \n{\n";
    for (const char* k : {"Gei_max", "Gie_max", "delay_constant"})
        o += std::string("\t") + k + " = " + fixed6(v("connectionParameters", k)) + ";\n";
    o += "};\n\n";
    std::ofstream f(path);
    f << o;
    return f ? UG_OK : ferr(UG_EIO, "cannot write " + path);
}

// ConfigurationNetworkTopology::write_configuration (ConfigurationNetworkTopology.cpp:64-82).
ug_status write_topology_cfg(const std::string& path, const Cfg& c)
{
    std::string arrangement;
    auto gi = c.groups.find("spatialParameters");
    if (gi != c.groups.end() && gi->second.count("arrangement")) arrangement = gi->second.at("arrangement");
    auto v = [&](const char* k) {
        double x = 0.0;
        c.num("spatialParameters", k, x);
        return x;
    };
    std::string o = "spatialParameters = \n{\n\tarrangement = \"" + arrangement + "\";\n";
    for (const char* k : {"A_RA2I", "SIGMA_RA2I", "B_I2RA", "SIGMA_I2RA"})
        o += std::string("\t") + k + " = " + fixed6(v(k)) + ";\n";
    o += "\n};\n\n";
    std::ofstream f(path);
    f << o;
    return f ? UG_OK : ferr(UG_EIO, "cannot write " + path);
}

double sphere_dist(const double* a, const double* b)
{
    const double t = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    return t > 1.0 ? 0.0 : std::acos(t);
}

}  // namespace

namespace {

// What new_chain_growth's set-up reads from a topology directory (read_network_topology,
// NetworkGrowthSimulator.cpp:2628-2650) plus the training neurons.
struct GrowthSetup {
    int32_t nra = 0, ni = 0;
    double model = 0.0;
    std::vector<double> ra_xyz, i_xyz;   // 3 per neuron
    Conn ri, ir;
    std::vector<int32_t> training;       // sorted
    Cfg t;                               // the topology parameters (network_parameters.cfg)
};

ug_status setup_growth_network(ug_ctx* ctx, GrowthSetup& su, const Cfg& g, const std::string& out_dir,
                               int32_t num_steps, uint64_t seed, int32_t stream_id, int32_t* net_id);

}  // namespace

extern "C" ug_status ug_create_growth_network(ug_ctx* ctx, const char* network_dir, const char* training_file,
                                              const char* config_file, const char* out_dir_c, int32_t num_steps,
                                              uint64_t seed, int32_t stream_id, int32_t* net_id)
{
    if (!ctx || !network_dir || !training_file || !config_file || !net_id) return ferr(UG_EINVAL, "null argument");
    const std::string dir(network_dir), out_dir(out_dir_c ? out_dir_c : "");
    Cfg g;
    GrowthSetup su;
    UG_FTRY(parse_cfg(config_file, g));
    UG_FTRY(parse_cfg(join(dir, "network_parameters.cfg"), su.t));
    {
        In in(join(dir, "num_neurons.bin"));
        if (!in.ok() || !in.get(su.nra) || !in.get(su.ni) || su.nra <= 0 || su.ni < 0) return bad_file(in);
    }
    double model_i = 0.0;
    UG_FTRY(read_coords(join(dir, "RA_xy.bin"), su.nra, su.ra_xyz, su.model));
    UG_FTRY(read_coords(join(dir, "I_xy.bin"), su.ni, su.i_xyz, model_i));
    UG_FTRY(read_connections(join(dir, "RA_I_connections.bin"), su.nra, su.ri.off, su.ri.tgt, su.ri.w, su.ri.len,
                             su.ri.d));
    UG_FTRY(read_connections(join(dir, "I_RA_connections.bin"), su.ni, su.ir.off, su.ir.tgt, su.ir.w, su.ir.len,
                             su.ir.d));
    {
        In in(training_file);
        int32_t k = 0;
        if (!in.ok() || !in.get(k) || k < 0 || !in.get(su.training, (size_t)k)) return bad_file(in);
    }
    return setup_growth_network(ctx, su, g, out_dir, num_steps, seed, stream_id, net_id);
}

extern "C" ug_status ug_create_growth_network_from_topology(ug_ctx* ctx, const ug_topology* topo, int32_t training_set,
                                                            const char* config_file, const char* out_dir_c,
                                                            int32_t num_steps, uint64_t seed, int32_t stream_id,
                                                            int32_t* net_id)
{
    if (!ctx || !topo || !config_file || !net_id) return ferr(UG_EINVAL, "null argument");
    if (training_set != 0 && training_set != 1) return ferr(UG_EINVAL, "training_set must be 0 (clustered) or 1 (random)");
    Cfg g;
    UG_FTRY(parse_cfg(config_file, g));
    GrowthSetup su;
    su.nra = topo->n_ra;
    su.ni = topo->n_i;
    su.model = topo->model;
    su.ra_xyz = topo->ra_xyz;
    su.i_xyz = topo->i_xyz;
    su.ri.off = topo->ri_off;
    su.ri.tgt = topo->ri_tgt;
    su.ri.len = topo->ri_len;
    su.ri.w.assign(topo->ri_tgt.size(), 0.0);
    su.ri.d.assign(topo->ri_tgt.size(), 0.0);
    su.ir.off = topo->ir_off;
    su.ir.tgt = topo->ir_tgt;
    su.ir.len = topo->ir_len;
    su.ir.w.assign(topo->ir_tgt.size(), 0.0);
    su.ir.d.assign(topo->ir_tgt.size(), 0.0);
    su.training = training_set == 0 ? topo->clustered : topo->random_set;
    // the topology parameters as network_parameters.cfg would hold them, at full precision
    auto& sp = su.t.groups["spatialParameters"];
    sp["arrangement"] = topo->params.arrangement == UG_ARRANGEMENT_SQUARE ? "square" : "sphere";
    const double vals[4] = {topo->params.A_RA2I, topo->params.SIGMA_RA2I, topo->params.B_I2RA, topo->params.SIGMA_I2RA};
    const char* keys[4] = {"A_RA2I", "SIGMA_RA2I", "B_I2RA", "SIGMA_I2RA"};
    for (int k = 0; k < 4; ++k) {
        char b[64];
        std::snprintf(b, sizeof(b), "%.17g", vals[k]);
        sp[keys[k]] = b;
    }
    return setup_growth_network(ctx, su, g, out_dir_c ? out_dir_c : "", num_steps, seed, stream_id, net_id);
}

namespace {

// The rest of new_chain_growth's set-up (NetworkGrowthSimulator.cpp:1865-1940) on what
// was read: delays from the lengths, the RA<->I weights redrawn, the training neurons made
// mature, the set-up files written into out_dir (when given), and the network loaded.
ug_status setup_growth_network(ug_ctx* ctx, GrowthSetup& su, const Cfg& g, const std::string& out_dir,
                               int32_t num_steps, uint64_t seed, int32_t stream_id, int32_t* net_id)
{
    const int32_t nra = su.nra, ni = su.ni;
    const double model = su.model;
    std::vector<double>& ra_xyz = su.ra_xyz;
    std::vector<double>& i_xyz = su.i_xyz;
    Conn& ri = su.ri;
    Conn& ir = su.ir;
    const Cfg& t = su.t;
    std::vector<int32_t>& training = su.training;
    std::sort(training.begin(), training.end());
    for (int32_t id : training)
        if (id < 0 || id >= nra) return ferr(UG_EINVAL, "training neuron out of range");
    double dc = 0.0, gei = 0.0, gie = 0.0;
    g.num("connectionParameters", "delay_constant", dc);
    g.num("connectionParameters", "Gei_max", gei);
    g.num("connectionParameters", "Gie_max", gie);
    if (!(model > 0.0)) return ferr(UG_EINVAL, "RA_xy.bin holds no model interneuron distance");
    // sample_axonal_delays: lengths on the sphere in microns (EXPERIMENTAL_INTERNEURON_DISTANCE 40),
    // 0.01 ms per micron times the delay constant
    std::vector<double> L((size_t)nra * nra, 0.0), D((size_t)nra * nra, 0.0);
    for (int i = 0; i < nra; ++i)
        for (int j = 0; j < nra; ++j) {
            const double len = j != i ? sphere_dist(&ra_xyz[3 * i], &ra_xyz[3 * j]) * 40.0 / model : 0.0;
            L[(size_t)i * nra + j] = len;
            D[(size_t)i * nra + j] = len * 0.01 * dc;
        }
    for (size_t k = 0; k < ri.len.size(); ++k) ri.d[k] = ri.len[k] * 0.01 * dc;
    for (size_t k = 0; k < ir.len.size(); ++k) ir.d[k] = ir.len[k] * 0.01 * dc;
    // resample_weights: I->RA first, then RA->I, uniform below the maxima
    ug::HostStream hs{ug::make_stream(seed, ug::kNoiseCreate, (uint32_t)stream_id, 0, 0), 0};
    for (double& w : ir.w) w = ug::random_G(1.0, hs.word()) * gie;
    for (double& w : ri.w) w = ug::random_G(1.0, hs.word()) * gei;
    // neuron state: immature and spontaneous, the training neurons mature
    double e_mat = 0, e_imm = 0, g_mat = 0, g_imm = 0, win_d = 0;
    g.num("maturationParameters", "E_REST_MATURE", e_mat);
    g.num("maturationParameters", "E_REST_IMMATURE", e_imm);
    g.num("maturationParameters", "GCA_MATURE", g_mat);
    g.num("maturationParameters", "GCA_IMMATURE", g_imm);
    g.num("maturationParameters", "RATE_WINDOW_LONG", win_d);
    const int win = (int)win_d;
    std::vector<double> rest(nra, e_imm), gca(nra, g_imm), scale(nra, 100000.0), spread(training.size(), 0.0);
    std::vector<int32_t> mature(nra, 0), remod(nra, 0), tar(nra, 0), hist((size_t)nra * std::max(win, 0), 0);
    for (int32_t id : training) {
        mature[id] = 1;
        gca[id] = g_mat;
        rest[id] = e_mat;
    }
    std::vector<double> W((size_t)nra * nra, 0.0);
    std::vector<int32_t> act_off(nra + 1, 0), sup_off(nra + 1, 0), empty(1, 0);
    // files new_chain_growth writes
    if (!out_dir.empty()) {
        UG_FTRY(write_topology_cfg(join(out_dir, "network_parameters.cfg"), t));
        UG_FTRY(write_growth_cfg(join(out_dir, "growth_parameters.cfg"), g));
        const std::string pi = join(out_dir, "I_xy.bin");
        Out oi(pi, false);
        write_coords(oi, ni, i_xyz, model);
        UG_FTRY(closed(oi, pi));
        const std::string pn = join(out_dir, "training_neurons.bin"), ps = join(out_dir, "training_spread.bin");
        Out on(pn, false), os(ps, false);
        on.put((int32_t)training.size());
        on.put(training.data(), training.size());
        os.put((int32_t)spread.size());
        os.put(spread.data(), spread.size());
        UG_FTRY(closed(on, pn));
        UG_FTRY(closed(os, ps));
        const std::string pnn = join(out_dir, "num_neurons.bin");
        Out onn(pnn, false);
        onn.put(nra); onn.put(ni);
        UG_FTRY(closed(onn, pnn));
        const std::string pr = join(out_dir, "RA_xy_initial.bin");
        Out orr(pr, false);
        write_coords(orr, nra, ra_xyz, model);
        UG_FTRY(closed(orr, pr));
        const std::string p1 = join(out_dir, "RA_I_connections_initial.bin"), p2 = join(out_dir, "I_RA_connections_initial.bin");
        Out a(p1, false), b(p2, false);
        write_connections(a, nra, ri.off, ri.tgt, ri.w, ri.len, ri.d);
        write_connections(b, ni, ir.off, ir.tgt, ir.w, ir.len, ir.d);
        UG_FTRY(closed(a, p1));
        UG_FTRY(closed(b, p2));
    }
    ug_network_desc d;
    std::memset(&d, 0, sizeof(d));
    d.n_ra = nra; d.n_i = ni;
    d.num_steps = num_steps > 0 ? num_steps : 25000;
    d.net_id = stream_id;
    d.seed = seed;
    auto num = [](const Cfg& c, const char* grp, const char* key) {
        double v = 0.0;
        c.num(grp, key, v);
        return v;
    };
    d.syn.Nss = (int32_t)num(g, "synapticParameters", "Nss");
    double* syn_vals[] = {&d.syn.A_P, &d.syn.A_D, &d.syn.T_0, &d.syn.T_P, &d.syn.T_D, &d.syn.TAU_P, &d.syn.TAU_D,
                          &d.syn.BETA, &d.syn.BETA_SUPERSYNAPSE, &d.syn.ACTIVATION_THRESHOLD,
                          &d.syn.SUPERSYNAPSE_THRESHOLD, &d.syn.WEIGHT_MAX};
    for (int k = 0; k < 12; ++k) *syn_vals[k] = num(g, "synapticParameters", kSynFields[k]);
    d.mat.E_REST_MATURE = e_mat; d.mat.E_REST_IMMATURE = e_imm; d.mat.GCA_MATURE = g_mat; d.mat.GCA_IMMATURE = g_imm;
    d.mat.DEATH_RATE_THRESHOLD = num(g, "maturationParameters", "DEATH_RATE_THRESHOLD");
    d.mat.RATE_WINDOW_LONG = win;
    d.noise.white_noise_mean_soma = num(g, "noiseParameters", "white_noise_mean_soma");
    d.noise.white_noise_std_soma = num(g, "noiseParameters", "white_noise_std_soma");
    d.noise.white_noise_mean_dend = num(g, "noiseParameters", "white_noise_mean_dend");
    d.noise.white_noise_std_dend = num(g, "noiseParameters", "white_noise_std_dend");
    d.conn.Gei_max = gei; d.conn.Gie_max = gie; d.conn.delay_constant = dc;
    d.conn.A_RA2I = num(t, "spatialParameters", "A_RA2I"); d.conn.SIGMA_RA2I = num(t, "spatialParameters", "SIGMA_RA2I");
    d.conn.B_I2RA = num(t, "spatialParameters", "B_I2RA"); d.conn.SIGMA_I2RA = num(t, "spatialParameters", "SIGMA_I2RA");
    d.conn.model_interneuron_distance = model;
    d.ra2i_off = ri.off.data(); d.ra2i_tgt = ri.tgt.data(); d.ra2i_w = ri.w.data(); d.ra2i_d = ri.d.data();
    d.ra2i_len = ri.len.data();
    d.i2ra_off = ir.off.data(); d.i2ra_tgt = ir.tgt.data(); d.i2ra_w = ir.w.data(); d.i2ra_d = ir.d.data();
    d.i2ra_len = ir.len.data();
    d.w_rara = W.data(); d.d_rara = D.data(); d.len_rara = L.data();
    d.active_off = act_off.data(); d.active_tgt = empty.data();
    d.super_off = sup_off.data(); d.super_tgt = empty.data();
    d.rest_potential = rest.data(); d.gca = gca.data();
    d.mature = mature.data(); d.maturation_scale = scale.data();
    d.remodeled = remod.data(); d.trials_after_replacement = tar.data();
    d.activity_history = hist.data();
    d.n_tr = (int32_t)training.size();
    d.training = training.data(); d.training_spread = spread.data();
    d.ra_xyz = ra_xyz.data(); d.i_xyz = i_xyz.data();
    return ug_load_network(ctx, &d, net_id);
}

}  // namespace

// ---------------------------------------------------------------- generated topologies

namespace {

// std::ostream's default rendering of a double (six significant digits)
std::string g6(double v)
{
    char b[64];
    std::snprintf(b, sizeof(b), "%g", v);
    return b;
}

}  // namespace

extern "C" ug_status ug_topology_write_dir(const ug_topology* t, const char* dir_c)
{
    if (!t || !dir_c) return ferr(UG_EINVAL, "null argument");
    const std::string dir(dir_c);
    const int dim = t->dim();
    // write_network_topology (:18294-18310)
    const std::string pi = join(dir, "I_xy.bin"), pr = join(dir, "RA_xy.bin");
    Out oi(pi, false), orr(pr, false);
    write_coords(oi, t->n_i, t->i_xyz, t->model, dim);
    write_coords(orr, t->n_ra, t->ra_xyz, t->model, dim);
    UG_FTRY(closed(oi, pi));
    UG_FTRY(closed(orr, pr));
    // write_connections_RAandI (:18312-18365): weights sample_G(0.0) = 0, delays 0
    const std::string p1 = join(dir, "RA_I_connections.bin"), p2 = join(dir, "I_RA_connections.bin");
    Out a(p1, false), b(p2, false);
    const std::vector<double> zri(t->ri_tgt.size(), 0.0), zir(t->ir_tgt.size(), 0.0);
    write_connections(a, t->n_ra, t->ri_off, t->ri_tgt, zri, t->ri_len, zri);
    write_connections(b, t->n_i, t->ir_off, t->ir_tgt, zir, t->ir_len, zir);
    UG_FTRY(closed(a, p1));
    UG_FTRY(closed(b, p2));
    const std::string pn = join(dir, "num_neurons.bin");
    Out on(pn, false);
    on.put((int32_t)t->n_ra);
    on.put((int32_t)t->n_i);
    UG_FTRY(closed(on, pn));
    // write_different_training_arrangements (:406-457)
    for (int which = 0; which < 2; ++which) {
        const std::string p = join(dir, which == 0 ? "training_neurons_clustered.bin" : "training_neurons_random.bin");
        const std::vector<int32_t>& v = which == 0 ? t->clustered : t->random_set;
        Out o(p, false);
        o.put((int32_t)v.size());
        o.put(v.data(), v.size());
        UG_FTRY(closed(o, p));
    }
    // write_pajek_topology (:18367-18429); the training neurons it marks are the random set,
    // the last one generate_network_topology assigned
    std::vector<char> training(t->n_ra, 0);
    for (int32_t id : t->random_set) training[id] = 1;
    std::string s = "*Vertices " + std::to_string(t->n_ra + t->n_i) + "\n";
    auto coords = [&](const std::vector<double>& xyz, int i) {
        std::string c = g6(xyz[3 * (size_t)i]) + " " + g6(xyz[3 * (size_t)i + 1]);
        if (dim == 3) c += " " + g6(xyz[3 * (size_t)i + 2]);
        return c;
    };
    for (int i = 0; i < t->n_ra; ++i)
        s += std::to_string(i + 1) + " \"" + std::to_string(i) + "\" " + coords(t->ra_xyz, i) +
             (training[i] ? " ic Yellow\n" : " ic Green\n");
    for (int i = 0; i < t->n_i; ++i)
        s += std::to_string(i + t->n_ra + 1) + " \"" + std::to_string(i + t->n_ra) + "\" " + coords(t->i_xyz, i) +
             " ic Red\n";
    s += "*Arcs\n";
    for (int i = 0; i < t->n_ra; ++i)
        for (int32_t k = t->ri_off[i]; k < t->ri_off[i + 1]; ++k)
            s += std::to_string(i + 1) + " " + std::to_string(t->ri_tgt[k] + t->n_ra + 1) + " " + g6(0.0) + " c Green\n";
    for (int i = 0; i < t->n_i; ++i)
        for (int32_t k = t->ir_off[i]; k < t->ir_off[i + 1]; ++k)
            s += std::to_string(i + t->n_ra + 1) + " " + std::to_string(t->ir_tgt[k] + 1) + " " + g6(0.0) + " c Red\n";
    const std::string pp = join(dir, "network_topology.net");
    std::ofstream f(pp);
    f << s;
    f.close();
    return f ? UG_OK : ferr(UG_EIO, "cannot write " + pp);
}

extern "C" ug_status ug_create_network_topology(ug_ctx* ctx, const char* config_file, const char* network_dir,
                                                int32_t n_ra, int32_t n_i, int32_t n_tr, uint64_t seed,
                                                ug_topology_info* info)
{
    if (!ctx || !config_file || !network_dir) return ferr(UG_EINVAL, "null argument");
    Cfg c;
    UG_FTRY(parse_cfg(config_file, c));
    ug_topology_params p;
    std::memset(&p, 0, sizeof(p));
    std::string arrangement;
    auto gi = c.groups.find("spatialParameters");
    if (gi != c.groups.end() && gi->second.count("arrangement")) arrangement = gi->second.at("arrangement");
    if (arrangement == "sphere")
        p.arrangement = UG_ARRANGEMENT_SPHERE;
    else if (arrangement == "square")
        p.arrangement = UG_ARRANGEMENT_SQUARE;
    else
        return ferr(UG_EINVAL, "arrangement \"" + arrangement + "\" is not generated (sphere or square)");
    c.num("spatialParameters", "A_RA2I", p.A_RA2I);
    c.num("spatialParameters", "SIGMA_RA2I", p.SIGMA_RA2I);
    c.num("spatialParameters", "B_I2RA", p.B_I2RA);
    c.num("spatialParameters", "SIGMA_I2RA", p.SIGMA_I2RA);
    ug_topology* t = nullptr;
    UG_FTRY(ug_generate_topology(ctx, &p, n_ra, n_i, n_tr, seed, 0, &t));
    const ug_status s = ug_topology_write_dir(t, network_dir);
    if (s == UG_OK && info) ug_topology_get_info(t, info);
    ug_topology_free(t);
    return s;
}
