// vcfpop-gb300: drop-in driver for vcfpop's -structure analysis on one GPU.
//
// Takes the reference's flag block (-g_input, -g_output, -g_seed, -g_indtext,
// -g_decimal, -g_delimiter, -g_linebreak and -structure_*,
// src/parameters.cpp:584-627, 1230-1307), reads VCF (plain or gzip), groups
// individuals by population as the reference does (src/filter.cpp:300-345),
// runs every (K, replicate) run through libvcfpop_structure and writes the
// reference's result files (src/structure.cpp:86-401):
//   <out>.structure.k=K_rep=R_id=I.txt, its .lnl.txt with -structure_writelnl,
//   and the summary <out>.structure.txt.
// Extra flags: -gb300_rng=counter|reference, -gb300_form=plain|tc|auto
// (auto, the default: the tensor-core form wherever it applies),
// -gb300_device=D. Filters of the reference that are not implemented are
// refused.
#include <zlib.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <map>
#include <string>
#include <vector>

#include "../../include/vcfpop_structure.h"

namespace {

struct Opts {
    std::string input, output = "vcfpop", indtext;
    int64_t seed = 0;
    int decimal = 5;
    std::string delim = "\t", lb = "\r\n";
    int kmin = 1, kmax = 5, nruns = 1, diversity = 0, device = 0;
    int form = -1;                // -gb300_form: VP_FORM_*, or -1 = tensor-core form where it applies
    bool filter = false;          // -f, with -f_* windows: the locus filter
    vp_locus_filter lf{};
    // the individual filter (-f_itype, -f_iploidy), applied before the locus filter
    bool itype_b = false, iploidy_b = false;
    double itype_min = 0, itype_max = 0;
    int iploidy_min = 0, iploidy_max = 0;
    vp_params p;
    std::vector<std::string> argv;
};

int yesno(const std::string& v) { return v == "yes" ? 1 : 0; }

bool parse(int argc, char** argv, Opts& o) {
    vp_params_default(&o.p);
    o.p.rng = VP_RNG_COUNTER;
    bool structure = false;
    std::vector<std::string> unimplemented;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        o.argv.push_back(a);
        size_t eq = a.find('=');
        std::string k = a.substr(0, eq), v = eq == std::string::npos ? "" : a.substr(eq + 1);
        if (v.size() >= 2 && v.front() == '"' && v.back() == '"') v = v.substr(1, v.size() - 2);
        if (k == "-structure") structure = true;
        else if (k == "-g_input") o.input = v;
        else if (k == "-g_output") o.output = v;
        else if (k == "-g_seed") o.seed = atoll(v.c_str());
        else if (k == "-g_decimal") o.decimal = atoi(v.c_str());
        else if (k == "-g_indtext") o.indtext = v;
        else if (k == "-g_delimiter") o.delim = v == "comma" ? "," : "\t";
        else if (k == "-g_linebreak") o.lb = v == "unix" ? "\n" : "\r\n";
        else if (k == "-gb300_rng") o.p.rng = v == "reference" ? VP_RNG_REFERENCE : VP_RNG_COUNTER;
        else if (k == "-gb300_form") o.form = v == "tc" ? VP_FORM_TC : v == "plain" ? VP_FORM_PLAIN : -1;
        else if (k == "-gb300_device") o.device = atoi(v.c_str());
        else if (k == "-structure_admix") o.p.admix = yesno(v);
        else if (k == "-structure_locpriori") o.p.locpriori = yesno(v);
        else if (k == "-structure_f") o.p.fmodel = yesno(v);
        else if (k == "-structure_krange") sscanf(v.c_str(), "[%d,%d]", &o.kmin, &o.kmax);
        else if (k == "-structure_nburnin") o.p.nburnin = atoi(v.c_str());
        else if (k == "-structure_nreps") o.p.nreps = atoi(v.c_str());
        else if (k == "-structure_nthinning") o.p.nthinning = atoi(v.c_str());
        else if (k == "-structure_nruns") o.nruns = atoi(v.c_str());
        else if (k == "-structure_nadmburnin") o.p.nadmburnin = atoi(v.c_str());
        else if (k == "-structure_writelnl") o.p.writelnl = yesno(v);
        else if (k == "-structure_diversity") o.diversity = yesno(v);
        else if (k == "-structure_lambda") o.p.lambda = atof(v.c_str());
        else if (k == "-structure_stdlambda") o.p.stdlambda = atof(v.c_str());
        else if (k == "-structure_maxlambda") o.p.maxlambda = atof(v.c_str());
        else if (k == "-structure_alpha") o.p.alpha = atof(v.c_str());
        else if (k == "-structure_inferalpha") o.p.inferalpha = yesno(v);
        else if (k == "-structure_diffalpha") o.p.diffalpha = yesno(v);
        else if (k == "-structure_uniformalpha") o.p.uniformalpha = yesno(v);
        else if (k == "-structure_stdalpha") o.p.stdalpha = atof(v.c_str());
        else if (k == "-structure_maxalpha") o.p.maxalpha = atof(v.c_str());
        else if (k == "-structure_alphapriora") o.p.alphapriora = atof(v.c_str());
        else if (k == "-structure_alphapriorb") o.p.alphapriorb = atof(v.c_str());
        else if (k == "-structure_metrofreq") o.p.metrofreq = atoi(v.c_str());
        else if (k == "-structure_r") o.p.r = atof(v.c_str());
        else if (k == "-structure_maxr") o.p.maxr = atof(v.c_str());
        else if (k == "-structure_stdr") o.p.epsr = atof(v.c_str());
        else if (k == "-structure_epseta") o.p.epseta = atof(v.c_str());
        else if (k == "-structure_epsgamma") o.p.epsgamma = atof(v.c_str());
        else if (k == "-structure_pmeanf") o.p.pmeanf = atof(v.c_str());
        else if (k == "-structure_pstdf") o.p.pstdf = atof(v.c_str());
        else if (k == "-structure_stdf") o.p.stdf = atof(v.c_str());
        else if (k == "-structure_singlef") o.p.fsame = yesno(v);
        else if (k == "-f") o.filter = true;
        else if (k == "-g_float") o.lf.single = v == "single";
        else if (k == "-f_bmaf") o.lf.bmaf_b = sscanf(v.c_str(), "[%lf,%lf]", &o.lf.bmaf_min, &o.lf.bmaf_max) == 2;
        else if (k == "-f_k") o.lf.k_b = sscanf(v.c_str(), "[%d,%d]", &o.lf.k_min, &o.lf.k_max) == 2;
        else if (k == "-f_n") o.lf.n_b = sscanf(v.c_str(), "[%d,%d]", &o.lf.n_min, &o.lf.n_max) == 2;
        else if (k == "-f_ptype") o.lf.ptype_b = sscanf(v.c_str(), "[%lf,%lf]", &o.lf.ptype_min, &o.lf.ptype_max) == 2;
        else if (k == "-f_he") o.lf.he_b = sscanf(v.c_str(), "[%lf,%lf]", &o.lf.he_min, &o.lf.he_max) == 2;
        else if (k == "-f_ho") o.lf.ho_b = sscanf(v.c_str(), "[%lf,%lf]", &o.lf.ho_min, &o.lf.ho_max) == 2;
        else if (k == "-f_pic") o.lf.pic_b = sscanf(v.c_str(), "[%lf,%lf]", &o.lf.pic_min, &o.lf.pic_max) == 2;
        else if (k == "-f_ae") o.lf.ae_b = sscanf(v.c_str(), "[%lf,%lf]", &o.lf.ae_min, &o.lf.ae_max) == 2;
        else if (k == "-f_I") o.lf.I_b = sscanf(v.c_str(), "[%lf,%lf]", &o.lf.I_min, &o.lf.I_max) == 2;
        else if (k == "-f_pval") o.lf.pval_b = sscanf(v.c_str(), "[%lf,%lf]", &o.lf.pval_min, &o.lf.pval_max) == 2;
        else if (k == "-f_itype") o.itype_b = sscanf(v.c_str(), "[%lf,%lf]", &o.itype_min, &o.itype_max) == 2;
        else if (k == "-f_iploidy") o.iploidy_b = sscanf(v.c_str(), "[%d,%d]", &o.iploidy_min, &o.iploidy_max) == 2;
        else if (k.rfind("-f_", 0) == 0) unimplemented.push_back(k);
        // other -g_* and -structure_* flags (threads, SIMD, plots, streams) do
        // not apply to the GPU path and are accepted silently
    }
    // the reference applies its -f_* windows only under -f
    // (src/parameters.cpp:1336-1343); every other filter of the reference
    // (-f_qual, -f_dp, -f_gq, -f_windowsize, ...) would change which
    // loci, calls or individuals the clustering sees: refuse it rather than
    // run on unfiltered data
    if (o.filter && !unimplemented.empty()) {
        fprintf(stderr, "vcfpop-gb300: the filter %s is not implemented (implemented: -f_bmaf -f_k -f_n -f_ptype "
                        "-f_he -f_ho -f_pic -f_ae -f_I -f_pval -f_itype -f_iploidy)\n", unimplemented[0].c_str());
        return false;
    }
    if (!structure) { fprintf(stderr, "vcfpop-gb300: only -structure is implemented\n"); return false; }
    if (o.input.empty()) { fprintf(stderr, "vcfpop-gb300: -g_input is required\n"); return false; }
    return true;
}

struct Vcf {
    std::vector<std::string> inds, locs;
    std::vector<int32_t> ploidy, k;
    std::vector<int8_t> G;  // [L][N][vmax]
    int vmax = 0;
};

bool read_vcf(const std::string& path, Vcf& v) {
    gzFile f = gzopen(path.c_str(), "rb");
    if (!f) return false;
    std::vector<char> buf(1 << 24);
    std::string line;
    int64_t nl = 0;
    auto getline_gz = [&](std::string& out) -> bool {
        out.clear();
        for (;;) {
            if (!gzgets(f, buf.data(), (int)buf.size())) return !out.empty();
            out += buf.data();
            if (!out.empty() && out.back() == '\n') return true;
        }
    };
    while (getline_gz(line)) {
        while (!line.empty() && (line.back() == '\n' || line.back() == '\r')) line.pop_back();
        if (line.rfind("##", 0) == 0) continue;
        std::vector<std::string> cols;
        size_t s0 = 0;
        for (;;) {
            size_t t = line.find('\t', s0);
            cols.push_back(line.substr(s0, t == std::string::npos ? std::string::npos : t - s0));
            if (t == std::string::npos) break;
            s0 = t + 1;
        }
        if (line[0] == '#') {
            for (size_t c = 9; c < cols.size(); ++c) v.inds.push_back(cols[c]);
            continue;
        }
        const int N = (int)v.inds.size();
        int nalt = 1;
        for (char ch : cols[4]) nalt += ch == ',';
        v.k.push_back(1 + nalt);
        // the reference's default locus name: CHROM_ID (CHROM_POS without an ID)
        v.locs.push_back(cols[0] + "_" + (cols[2] != "." ? cols[2] : cols[1]));
        if (nl == 0) {
            for (int i = 0; i < N; ++i) {
                const std::string& g = cols[9 + i];
                int p = 1;
                for (char ch : g.substr(0, g.find(':'))) p += ch == '/' || ch == '|';
                v.ploidy.push_back(p);
                v.vmax = std::max(v.vmax, p);
            }
        }
        size_t base = v.G.size();
        v.G.resize(base + (size_t)N * v.vmax, -1);
        for (int i = 0; i < N; ++i) {
            std::string g = cols[9 + i];
            g = g.substr(0, g.find(':'));
            int8_t al[16];
            int n = 0;
            bool miss = false;
            size_t q = 0;
            while (q <= g.size() && n < 16) {
                size_t e = g.find_first_of("/|", q);
                std::string tok = g.substr(q, e == std::string::npos ? std::string::npos : e - q);
                if (tok == "." || tok.empty()) miss = true;
                else al[n] = (int8_t)atoi(tok.c_str());
                n++;
                if (e == std::string::npos) break;
                q = e + 1;
            }
            if (miss) continue;
            std::sort(al, al + n);
            for (int c = 0; c < n && c < v.vmax; ++c) v.G[base + (size_t)i * v.vmax + c] = al[c];
        }
        nl++;
    }
    gzclose(f);
    return nl > 0;
}

// The whole file in memory (gzip or plain), then its genotypes parsed on the
// device: into the 2-bit matrix (vp_vcf_pack2) for biallelic diploid data
// (returns 1), else into allele copies per call (vp_vcf_parse, returns 2).
// Returns 0 when the host reader has to take over.
int read_vcf_device(const Opts& o, Vcf& v, std::vector<uint32_t>& packed) {
    gzFile f = gzopen(o.input.c_str(), "rb");
    if (!f) return 0;
    std::vector<char> text;
    size_t n = 0;
    text.resize(1 << 26);
    for (;;) {
        if (text.size() - n < (1u << 24)) text.resize(text.size() * 2);
        int got = gzread(f, text.data() + n, (unsigned)std::min<size_t>(text.size() - n, 1u << 30));
        if (got <= 0) break;
        n += (size_t)got;
    }
    gzclose(f);
    // header: skip ## lines, take the sample names of the #CHROM line
    size_t p = 0;
    while (p < n && text[p] == '#' && p + 1 < n && text[p + 1] == '#') {
        const char* e = (const char*)memchr(text.data() + p, '\n', n - p);
        if (!e) return 0;
        p = (size_t)(e - text.data()) + 1;
    }
    if (p >= n || text[p] != '#') return 0;
    const char* he = (const char*)memchr(text.data() + p, '\n', n - p);
    if (!he) return 0;
    std::string hdr(text.data() + p, he - (text.data() + p));
    while (!hdr.empty() && hdr.back() == '\r') hdr.pop_back();
    int col = 0;
    size_t s0 = 0;
    for (;;) {
        size_t t = hdr.find('\t', s0);
        if (col >= 9) v.inds.push_back(hdr.substr(s0, t == std::string::npos ? std::string::npos : t - s0));
        ++col;
        if (t == std::string::npos) break;
        s0 = t + 1;
    }
    const int N = (int)v.inds.size();
    if (N == 0) return 0;
    const char* data = he + 1;
    const size_t bytes = n - (size_t)(data - text.data());
    int64_t L = 0;
    for (const char* q = data; (q = (const char*)memchr(q, '\n', bytes - (q - data))); ++q) ++L;
    if (bytes && data[bytes - 1] != '\n') ++L;
    if (L == 0) return 0;
    const int Nw = (N + 15) / 16;
    packed.assign((size_t)L * Nw, 0);
    std::vector<int64_t> starts(L + 1);
    int64_t got = 0;
    if (vp_vcf_pack2(data, bytes, N, o.device, packed.data(), L, starts.data(), &got) || got != L) {
        // not biallelic diploid: the general parse on the device (any ploidy
        // and allele count), with each sample's ploidy from its first call
        fprintf(stderr, "vcfpop-gb300: packed ingest not used (%s)\n", vp_last_error());
        packed.clear();
        int vmax = 1;
        {
            const char* le = (const char*)memchr(data, '\n', bytes);
            std::string first(data, le ? le - data : bytes);
            int field = 0, cur = 1;
            bool gt = false;
            for (char ch : first) {
                if (ch == '\t') { if (field >= 9) vmax = std::max(vmax, cur); ++field; cur = 1; gt = field >= 9; continue; }
                if (ch == ':') gt = false;
                if (gt && (ch == '/' || ch == '|')) ++cur;
            }
            if (field >= 9) vmax = std::max(vmax, cur);
        }
        vmax = std::min(vmax, 16);
        v.G.assign((size_t)L * N * vmax, -1);
        v.k.assign(L, 0);
        v.ploidy.assign(N, 0);
        if (vp_vcf_parse(data, bytes, N, vmax, o.device, v.G.data(), v.k.data(), v.ploidy.data(), L, starts.data(),
                         &got) || got != L) {
            fprintf(stderr, "vcfpop-gb300: device ingest not used (%s); reading on the host\n", vp_last_error());
            v = Vcf();
            return 0;
        }
        v.vmax = vmax;
        v.locs.resize(L);
        for (int64_t l = 0; l < L; ++l) {
            const char* a = data + starts[l];
            const char* e = data + starts[l + 1];
            const char* t1 = (const char*)memchr(a, '\t', e - a);
            const char* t2 = t1 ? (const char*)memchr(t1 + 1, '\t', e - t1 - 1) : nullptr;
            const char* t3 = t2 ? (const char*)memchr(t2 + 1, '\t', e - t2 - 1) : nullptr;
            if (!t1 || !t2 || !t3) { v = Vcf(); return 0; }
            std::string id(t2 + 1, t3 - t2 - 1);
            v.locs[l] = std::string(a, t1 - a) + "_" + (id != "." ? id : std::string(t1 + 1, t2 - t1 - 1));
        }
        return 2;
    }
    v.vmax = 2;
    v.ploidy.assign(N, 2);
    v.k.assign(L, 2);
    v.locs.resize(L);
    for (int64_t l = 0; l < L; ++l) {
        // CHROM_ID, or CHROM_POS without an ID (the reference's default locus name)
        const char* a = data + starts[l];
        const char* e = data + starts[l + 1];
        const char* t1 = (const char*)memchr(a, '\t', e - a);
        const char* t2 = t1 ? (const char*)memchr(t1 + 1, '\t', e - t1 - 1) : nullptr;
        const char* t3 = t2 ? (const char*)memchr(t2 + 1, '\t', e - t2 - 1) : nullptr;
        if (!t1 || !t2 || !t3) { v = Vcf(); packed.clear(); return 0; }
        std::string id(t2 + 1, t3 - t2 - 1);
        v.locs[l] = std::string(a, t1 - a) + "_" + (id != "." ? id : std::string(t1 + 1, t2 - t1 - 1));
    }
    return 1;
}

// -g_indtext="pop1:#1-#30,#40 pop2:#31-#39 ..." (1-based individual ranges)
void populations(const std::string& spec, int N, std::vector<int>& popid, std::vector<std::string>& names) {
    popid.assign(N, -1);
    if (spec.empty()) { names = {"pop1"}; popid.assign(N, 0); return; }
    size_t s0 = 0;
    while (s0 < spec.size()) {
        size_t e = spec.find(' ', s0);
        std::string tok = spec.substr(s0, e == std::string::npos ? std::string::npos : e - s0);
        s0 = e == std::string::npos ? spec.size() : e + 1;
        size_t colon = tok.find(':');
        if (colon == std::string::npos) continue;
        int pid = (int)names.size();
        names.push_back(tok.substr(0, colon));
        std::string r = tok.substr(colon + 1);
        size_t q = 0;
        while (q < r.size()) {
            size_t c = r.find(',', q);
            std::string rg = r.substr(q, c == std::string::npos ? std::string::npos : c - q);
            q = c == std::string::npos ? r.size() : c + 1;
            int a = 0, b = 0;
            if (sscanf(rg.c_str(), "#%d-#%d", &a, &b) != 2) { sscanf(rg.c_str(), "#%d", &a); b = a; }
            for (int i = a; i <= b && i <= N; ++i)
                if (i >= 1) popid[i - 1] = pid;
        }
    }
    // individuals without a population go to an extra "pop0"-style group at the end
    bool orphan = false;
    for (int i = 0; i < N; ++i)
        if (popid[i] < 0) { popid[i] = (int)names.size(); orphan = true; }
    if (orphan) names.push_back("Unassigned");
}

struct Writer {
    FILE* f;
    const Opts& o;
    char fmt[16];
    Writer(FILE* f_, const Opts& o_) : f(f_), o(o_) { snprintf(fmt, sizeof fmt, "%%0.%df", o.decimal); }
    void real(double v) {
        if (std::isnan(v) || std::isinf(v)) fputs("nan", f);
        else fprintf(f, fmt, v);
    }
    void s(const char* t) { fputs(t, f); }
    void lb() { fputs(o.lb.c_str(), f); }
    void d() { fputs(o.delim.c_str(), f); }
};

// The individual filter (MarkerIndividual and RemoveIndividual,
// src/filter.cpp:398-475 and 565-605), which the reference applies before the
// locus filter. -f_itype: an individual is removed when its count of typed
// loci lies outside (int64)(min * L + 0.5) .. (int64)(max * L + 0.5).
// -f_iploidy: the reference compares the window with the smallest and the
// largest ploidy over all individuals (the globals minploidy and maxploidy;
// an individual without any typed call counts as ploidy 0), not with each
// individual's own, so either every individual passes or every one is
// removed, which the reference reports as an error; that is reproduced.
bool individual_filter(const Opts& o, Vcf& v, bool dev_ingest, std::vector<uint32_t>& packed, std::vector<int>& pop) {
    const int N = (int)v.inds.size();
    const int64_t L = (int64_t)v.k.size();
    const int Nw = (N + 15) / 16;
    std::vector<int64_t> ntype(N, 0);
    std::vector<int> vmin(N, 100), vmax(N, 0);
    for (int64_t l = 0; l < L; ++l)
        for (int i = 0; i < N; ++i) {
            bool typed;
            if (dev_ingest) typed = ((packed[(size_t)l * Nw + (i >> 4)] >> (2 * (i & 15))) & 3u) != 3u;
            else typed = v.G[((size_t)l * N + i) * v.vmax] >= 0;
            if (typed) {
                ntype[i]++;
                vmin[i] = std::min(vmin[i], v.ploidy[i]);
                vmax[i] = std::max(vmax[i], v.ploidy[i]);
            }
        }
    int minploidy = 100, maxploidy = 0;
    for (int i = 0; i < N; ++i) {
        minploidy = std::min(minploidy, vmin[i] == 100 ? 0 : vmin[i]);
        maxploidy = std::max(maxploidy, vmax[i]);
    }
    const int64_t tmin = (int64_t)(o.itype_min * L + 0.5), tmax = (int64_t)(o.itype_max * L + 0.5);
    std::vector<int> keep;
    for (int i = 0; i < N; ++i) {
        bool pass = true;
        if (o.itype_b && (tmin > ntype[i] || ntype[i] > tmax)) pass = false;
        if (o.iploidy_b && (o.iploidy_min > minploidy || minploidy > o.iploidy_max)) pass = false;
        if (o.iploidy_b && (o.iploidy_min > maxploidy || maxploidy > o.iploidy_max)) pass = false;
        if (pass) keep.push_back(i);
    }
    if (keep.empty()) {
        fprintf(stderr, "vcfpop-gb300: all %d individuals are excluded from the analysis by the individual filter\n", N);
        return false;
    }
    fprintf(stderr, "vcfpop-gb300: individual filter kept %d of %d individuals\n", (int)keep.size(), N);
    if ((int)keep.size() == N) return true;
    const int M = (int)keep.size(), Mw = (M + 15) / 16;
    std::vector<std::string> inds(M);
    std::vector<int32_t> ploidy(M);
    std::vector<int> pp(M);
    for (int j = 0; j < M; ++j) { inds[j] = v.inds[keep[j]]; ploidy[j] = v.ploidy[keep[j]]; pp[j] = pop[keep[j]]; }
    if (dev_ingest) {
        std::vector<uint32_t> np((size_t)L * Mw, 0);
        for (int64_t l = 0; l < L; ++l)
            for (int j = 0; j < Mw * 16; ++j) {
                uint32_t code = 3;
                if (j < M) code = (packed[(size_t)l * Nw + (keep[j] >> 4)] >> (2 * (keep[j] & 15))) & 3u;
                np[(size_t)l * Mw + (j >> 4)] |= code << (2 * (j & 15));
            }
        packed.swap(np);
    } else {
        std::vector<int8_t> G((size_t)L * M * v.vmax);
        for (int64_t l = 0; l < L; ++l)
            for (int j = 0; j < M; ++j)
                memcpy(&G[((size_t)l * M + j) * v.vmax], &v.G[((size_t)l * N + keep[j]) * v.vmax], v.vmax);
        v.G.swap(G);
    }
    v.inds.swap(inds);
    v.ploidy.swap(ploidy);
    pop.swap(pp);
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    Opts o;
    if (!parse(argc, argv, o)) return 2;
    Vcf v;
    std::vector<uint32_t> dev_packed;   // device-parsed 2-bit matrix, file order of individuals
    const int ingest = read_vcf_device(o, v, dev_packed);
    const bool dev_ingest = ingest == 1;   // the 2-bit matrix (else allele copies in v.G)
    if (!ingest && !read_vcf(o.input, v)) { fprintf(stderr, "vcfpop-gb300: cannot read %s\n", o.input.c_str()); return 2; }
    const int N0 = (int)v.inds.size();
    const int64_t L0 = (int64_t)v.k.size();
    std::vector<int> pop;
    std::vector<std::string> pnames;
    populations(o.indtext, N0, pop, pnames);
    if (o.filter && (o.itype_b || o.iploidy_b)) {
        if (!individual_filter(o, v, dev_ingest, dev_packed, pop)) return 1;
    }
    const int N = (int)v.inds.size();
    // group individuals by population in the populations' order (stable)
    std::vector<int> perm(N);
    for (int i = 0; i < N; ++i) perm[i] = i;
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return pop[a] < pop[b]; });
    std::vector<std::string> inds(N);
    std::vector<int32_t> ploidy(N), popid(N);
    std::vector<int8_t> G(dev_ingest ? 0 : (size_t)L0 * N * v.vmax);
    bool identity = true;
    for (int j = 0; j < N; ++j) {
        int i = perm[j];
        identity &= i == j;
        inds[j] = v.inds[i]; ploidy[j] = v.ploidy[i]; popid[j] = pop[i];
        if (!dev_ingest)
            for (int64_t l = 0; l < L0; ++l)
                memcpy(&G[((size_t)l * N + j) * v.vmax], &v.G[((size_t)l * N + i) * v.vmax], v.vmax);
    }
    // drop populations without individuals, keeping the order
    std::vector<int> remap(pnames.size(), -1);
    std::vector<std::string> pn;
    for (int j = 0; j < N; ++j)
        if (remap[popid[j]] < 0) { remap[popid[j]] = (int)pn.size(); pn.push_back(pnames[popid[j]]); }
    for (int j = 0; j < N; ++j) popid[j] = remap[popid[j]];
    const int S = (int)pn.size();
    bool biallelic_diploid = v.vmax == 2;
    for (int i = 0; i < N && biallelic_diploid; ++i) biallelic_diploid = ploidy[i] == 2;
    for (int64_t l = 0; l < L0 && biallelic_diploid; ++l) biallelic_diploid = v.k[l] == 2;
    std::vector<uint32_t> packed;
    vp_input in{};
    in.n_ind = N; in.n_loc = L0; in.vmax = v.vmax; in.ploidy = ploidy.data(); in.n_alleles = v.k.data();
    in.popid = popid.data(); in.n_pop = S;
    if (dev_ingest && identity) {
        in.packed2 = dev_packed.data();
    } else if (dev_ingest) {
        // regroup the individuals of the device-parsed matrix by population
        const int Nw = (N + 15) / 16;
        packed.assign((size_t)L0 * Nw, 0);
        for (int64_t l = 0; l < L0; ++l) {
            const uint32_t* src = &dev_packed[(size_t)l * Nw];
            uint32_t* dst = &packed[(size_t)l * Nw];
            for (int j = 0; j < Nw * 16; ++j) {
                uint32_t code = 3;
                if (j < N) code = (src[perm[j] >> 4] >> (2 * (perm[j] & 15))) & 3u;
                dst[j >> 4] |= code << (2 * (j & 15));
            }
        }
        in.packed2 = packed.data();
    } else if (biallelic_diploid) {
        const int Nw = (N + 15) / 16;
        packed.assign((size_t)L0 * Nw, 0);
        for (int64_t l = 0; l < L0; ++l)
            for (int i = 0; i < Nw * 16; ++i) {
                int code = 3;
                if (i < N) {
                    const int8_t* g = &G[((size_t)l * N + i) * 2];
                    if (g[0] >= 0) code = g[0] + g[1];
                }
                packed[(size_t)l * Nw + i / 16] |= (uint32_t)code << (2 * (i % 16));
            }
        in.packed2 = packed.data();
    } else {
        in.alleles = G.data();
    }
    // the locus filter (-f with -f_* windows: src/filter.cpp MarkerDiversity)
    // on the packed matrix, on the device; loci that fail are dropped here
    const vp_locus_filter& lf = o.lf;
    const bool windows = lf.bmaf_b || lf.k_b || lf.n_b || lf.ptype_b || lf.he_b || lf.ho_b || lf.pic_b || lf.ae_b ||
                         lf.I_b || lf.pval_b;
    std::vector<uint32_t> kept_packed;
    if (o.filter && windows) {
        if (!in.packed2) { fprintf(stderr, "vcfpop-gb300: the locus filter needs biallelic diploid data\n"); return 1; }
        const int Nw = (N + 15) / 16;
        std::vector<uint8_t> keep(L0);
        if (vp_locus_filter_pack2(in.packed2, L0, N, &lf, o.device, keep.data(), nullptr)) {
            fprintf(stderr, "vcfpop-gb300: %s\n", vp_last_error());
            return 1;
        }
        int64_t nk = 0;
        for (int64_t l = 0; l < L0; ++l) nk += keep[l];
        kept_packed.resize((size_t)nk * Nw);
        std::vector<int32_t> k2;
        std::vector<std::string> locs2;
        for (int64_t l = 0, j = 0; l < L0; ++l)
            if (keep[l]) {
                memcpy(&kept_packed[(size_t)j++ * Nw], in.packed2 + (size_t)l * Nw, (size_t)Nw * 4);
                k2.push_back(v.k[l]);
                locs2.push_back(v.locs[l]);
            }
        v.k.swap(k2);
        v.locs.swap(locs2);
        in.packed2 = kept_packed.data();
        in.n_loc = nk;
        in.n_alleles = v.k.data();
        fprintf(stderr, "vcfpop-gb300: locus filter kept %lld of %lld loci\n", (long long)nk, (long long)L0);
    }
    vp_dataset* ds = nullptr;
    if (vp_dataset_prepare(&in, &ds)) { fprintf(stderr, "vcfpop-gb300: %s\n", vp_last_error()); return 1; }
    vp_dataset_info info;
    vp_dataset_info_get(ds, &info);
    vp_ctx* ctx = nullptr;
    if (vp_open(ds, o.device, &ctx)) { fprintf(stderr, "vcfpop-gb300: %s\n", vp_last_error()); return 1; }
    // the tensor-core K-sweep runs no-admixture chains without location
    // prior or F model, with counter streams, on biallelic diploid data; the
    // default picks it for every run where it applies (the no-admixture
    // burn-in runs in the plain form first)
    if (o.form >= 0) o.p.form = o.form;
    else o.p.form = !o.p.admix && !o.p.locpriori && !o.p.fmodel && o.p.rng == VP_RNG_COUNTER && info.packed2
                        ? VP_FORM_TC : VP_FORM_PLAIN;
    fprintf(stderr, "vcfpop-gb300: %s form\n", o.p.form == VP_FORM_TC ? "tensor-core" : "plain");
    struct Run { int K, rep, id; vp_chain* c; };
    std::vector<Run> runs;
    int id = 0;
    for (int K = o.kmin; K <= o.kmax; ++K)
        for (int rep = 1; rep <= o.nruns; ++rep) {
            ++id;
            vp_params p = o.p;
            p.K = K;
            p.seed = vp_run_seed(o.seed, id);
            vp_chain* c = nullptr;
            if (vp_chain_create(ctx, &p, &c)) { fprintf(stderr, "vcfpop-gb300: %s\n", vp_last_error()); return 1; }
            runs.push_back({K, rep, id, c});
        }
    std::vector<vp_chain*> cs;
    for (auto& r : runs) cs.push_back(r.c);
    if (vp_finish(cs.data(), (int)cs.size())) { fprintf(stderr, "vcfpop-gb300: %s\n", vp_last_error()); return 1; }
    // the run files through the library's writer (WriteStructure), from each
    // chain's device state
    std::vector<const char*> ind_c, pop_c, loc_c;
    for (auto& n : inds) ind_c.push_back(n.c_str());
    for (auto& n : pn) pop_c.push_back(n.c_str());
    for (auto& n : v.locs) loc_c.push_back(n.c_str());
    vp_write_opts wo{};
    wo.prefix = o.output.c_str();
    wo.ind_names = ind_c.data(); wo.pop_names = pop_c.data(); wo.loc_names = loc_c.data();
    wo.decimal = o.decimal; wo.comma = o.delim == ","; wo.unix_lb = o.lb == "\n"; wo.diversity = o.diversity;
    std::vector<std::array<double, 3>> table;
    for (auto& run : runs) {
        wo.rep = run.rep;
        wo.id = run.id;
        if (vp_write_structure(run.c, &wo)) { fprintf(stderr, "vcfpop-gb300: %s\n", vp_last_error()); return 1; }
        vp_result r;
        vp_chain_sizes(run.c, &r);
        std::vector<double> rout(r.rlen);
        vp_result q{};
        q.rout = rout.data();
        if (vp_chain_result(run.c, &q)) { fprintf(stderr, "vcfpop-gb300: %s\n", vp_last_error()); return 1; }
        table.push_back({rout[0], rout[2], rout[3]});
        vp_chain_destroy(run.c);
    }
    // summary (src/structure.cpp:379-401)
    char fn[8192];
    snprintf(fn, sizeof fn, "%s.structure.txt", o.output.c_str());
    FILE* f = fopen(fn, "wb");
    Writer w(f, o);
    time_t now = time(nullptr);
    char tb[64];
    strftime(tb, sizeof tb, "%Y-%m-%d %H:%M:%S", localtime(&now));
    w.s("##Bayesian clustering calculated by vcfpop-gb300 (vcfpop v1.08b -structure)"); w.lb();
    w.s("#  Input: "); w.s(o.input.c_str()); w.lb();
    w.s("#  Output: "); w.s(o.output.c_str()); w.lb();
    w.s("#  Time: "); w.s(tb); w.lb();
    w.s("#  Parameter: "); w.s(argv[0]); w.lb();
    for (auto& a : o.argv) { w.s("#    "); w.s(a.c_str()); w.lb(); }
    w.lb(); w.lb(); w.s("ID"); w.d(); w.s("k"); w.d(); w.s("rep"); w.d(); w.s("Mean lnL"); w.d(); w.s("Var lnL"); w.d(); w.s("lnP(D)");
    for (size_t i = 0; i < runs.size(); ++i) {
        w.lb(); fprintf(f, "%d", runs[i].id); w.d(); fprintf(f, "%d", runs[i].K); w.d(); fprintf(f, "%d", runs[i].rep); w.d();
        w.real(table[i][0]); w.d(); w.real(table[i][1]); w.d(); w.real(table[i][2]);
    }
    fclose(f);
    vp_close(ctx);
    vp_dataset_free(ds);
    return 0;
}
