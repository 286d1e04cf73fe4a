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
#include "vp_callfilter.h"

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
    // the genotype filter (-f_dp, -f_gq, -f_ploidy), applied as the calls are read
    vp_call_filter cf{};
    // the locus filters on the VCF's fixed columns (-f_type, -f_original,
    // -f_chrprefix, -f_chrname; -f_qual is accepted and, as in the
    // reference, removes nothing) and the window filter (-f_windowsize,
    // -f_windowstat)
    int type_val = 0;                  // 1 snp, 2 indel, 3 both
    bool original_b = false;           // -f_original=yes
    bool chrprefix_b = false, chrname_b = false;
    std::vector<std::string> chrprefix, chrname;
    int64_t windowsize = 0;            // 0: no window filter
    int model_val = 0;                 // -f_model: 0 not given, 1 rcs, 2 prcs, 3 ces, 4 pes
    int windowstat = 5;                // 1 bmaf, 2 k, 3 n, 4 ptype, 5 he, 6 ho, 7 pic, 8 ae
    vp_params p;
    std::vector<std::string> argv;
};

int yesno(const std::string& v) { return v == "yes" ? 1 : 0; }

// a comma-separated list (SplitStr of TrimParQuote, src/parameters.cpp:703-714)
std::vector<std::string> split_list(const std::string& v) {
    std::vector<std::string> out;
    size_t q = 0;
    for (;;) {
        size_t c = v.find(',', q);
        out.push_back(v.substr(q, c == std::string::npos ? std::string::npos : c - q));
        if (c == std::string::npos) break;
        q = c + 1;
    }
    return out;
}

// the 1-based index of v in a '|' list of choices (GetParString), 0 if absent
int choice(const std::string& v, const char* list) {
    int idx = 1;
    std::string l(list);
    size_t q = 0;
    for (;;) {
        size_t c = l.find('|', q);
        if (l.substr(q, c == std::string::npos ? std::string::npos : c - q) == v) return idx;
        if (c == std::string::npos) return 0;
        q = c + 1;
        ++idx;
    }
}

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
        else if (k == "-f_dp" || k == "-f_gq" || k == "-f_ploidy") {
            // windows and ranges of GetRangeParInteger (src/parameters.cpp:743-748)
            int lo = 0, hi = 0;
            const int bound = k == "-f_dp" ? 0x7FFFFFFF : k == "-f_gq" ? 100 : 10, floor_ = k == "-f_ploidy" ? 1 : 0;
            if (sscanf(v.c_str(), "[%d,%d]", &lo, &hi) != 2 || lo < floor_ || hi > bound || lo > hi) {
                fprintf(stderr, "vcfpop-gb300: parameter %s out of range (%d to %d)\n", a.c_str(), floor_, bound);
                return false;
            }
            int32_t* w = k == "-f_dp" ? &o.cf.dp_b : k == "-f_gq" ? &o.cf.gq_b : &o.cf.ploidy_b;
            w[0] = 1; w[1] = lo; w[2] = hi;
        } else if (k == "-f_qual") {
            // the reference's test (qual < min && qual > max, src/load.cpp
            // :1916, 2420) never fails a locus for min <= max: only the
            // window is checked
            double lo = 0, hi = 0;
            if (sscanf(v.c_str(), "[%lf,%lf]", &lo, &hi) != 2 || lo < 0 || hi > 255 || lo > hi) {
                fprintf(stderr, "vcfpop-gb300: parameter %s out of range (0 to 255)\n", a.c_str());
                return false;
            }
        } else if (k == "-f_model") {
            // the genotype model of the HWE test, the same for every model
            // at ploidy 2 (the locus statistics here are for diploid data)
            if (!(o.model_val = choice(v, "rcs|prcs|ces|pes"))) { fprintf(stderr, "vcfpop-gb300: bad %s\n", a.c_str()); return false; }
        } else if (k == "-f_type") {
            if (!(o.type_val = choice(v, "snp|indel|both"))) { fprintf(stderr, "vcfpop-gb300: bad %s\n", a.c_str()); return false; }
        } else if (k == "-f_original") {
            const int c = choice(v, "yes|no");
            if (!c) { fprintf(stderr, "vcfpop-gb300: bad %s\n", a.c_str()); return false; }
            o.original_b = c == 1;
        } else if (k == "-f_chrprefix") { o.chrprefix_b = true; o.chrprefix = split_list(v); }
        else if (k == "-f_chrname") { o.chrname_b = true; o.chrname = split_list(v); }
        else if (k == "-f_windowsize") {
            o.windowsize = atoll(v.c_str());
            if (o.windowsize < 1 || o.windowsize > 1000000000) { fprintf(stderr, "vcfpop-gb300: bad %s\n", a.c_str()); return false; }
        } else if (k == "-f_windowstat") {
            if (!(o.windowstat = choice(v, "bmaf|k|n|ptype|he|ho|pic|ae"))) { fprintf(stderr, "vcfpop-gb300: bad %s\n", a.c_str()); return false; }
        } else if (k.rfind("-f_", 0) == 0) unimplemented.push_back(k);
        // other -g_* and -structure_* flags (threads, SIMD, plots, streams) do
        // not apply to the GPU path and are accepted silently
    }
    // the reference applies its -f_* filters only under -f
    // (src/parameters.cpp:1336-1343); a filter of the reference that is not
    // implemented here (-f_pop) would change which loci the clustering sees:
    // refuse it rather than run on unfiltered data
    if (o.filter && !unimplemented.empty()) {
        fprintf(stderr, "vcfpop-gb300: the filter %s is not implemented (implemented: -f_bmaf -f_k -f_n -f_ptype "
                        "-f_he -f_ho -f_pic -f_ae -f_I -f_pval -f_itype -f_iploidy -f_dp -f_gq -f_ploidy -f_qual "
                        "-f_model -f_type -f_original -f_chrprefix -f_chrname -f_windowsize -f_windowstat)\n",
                unimplemented[0].c_str());
        return false;
    }
    if (!o.filter) o.cf = vp_call_filter{};
    if (!structure) { fprintf(stderr, "vcfpop-gb300: only -structure is implemented\n"); return false; }
    if (o.input.empty()) { fprintf(stderr, "vcfpop-gb300: -g_input is required\n"); return false; }
    return true;
}

struct Vcf {
    std::vector<std::string> inds, locs;
    std::vector<int32_t> ploidy, k;
    std::vector<int8_t> G;  // [L][N][vmax]
    int vmax = 0;
    // per locus: CHROM, POS, whether REF and the ALT alleles differ in
    // length (an indel, LOCUS::LOCUS src/function.cpp:3244-3253), whether
    // FILTER starts with "pass" in any case (src/load.cpp:2429-2434)
    std::vector<std::string> chrom;
    std::vector<int64_t> pos;
    std::vector<uint8_t> indel, pass;
};

// the fixed fields of one data line [a, e) into v's per-locus vectors;
// false when the line has fewer than 8 of them
bool line_info(const char* a, const char* e, Vcf& v) {
    const char* f[9];
    int n = 0;
    f[n++] = a;
    for (const char* q = a; q < e && n < 9; ++q)
        if (*q == '\t') f[n++] = q + 1;
    if (n < 8) return false;
    v.chrom.emplace_back(f[0], f[1] - 1 - f[0]);
    v.pos.push_back(strtoll(f[1], nullptr, 10));
    // allele string lengths: REF, then each comma-separated ALT
    int64_t mn = f[4] - 1 - f[3], mx = mn, cur = 0;
    for (const char* q = f[4]; q < f[5] - 1; ++q) {
        if (*q == ',') { mn = std::min(mn, cur); mx = std::max(mx, cur); cur = 0; }
        else ++cur;
    }
    mn = std::min(mn, cur);
    mx = std::max(mx, cur);
    v.indel.push_back(mn != mx);
    static const char kPass[] = "pass";
    bool pass = true;
    for (int j = 0; j < 4; ++j) {
        const char c = f[6] + j < e ? f[6][j] : '\0';
        if ((c >= 'A' && c <= 'Z' ? c + 32 : c) != kPass[j]) { pass = false; break; }
    }
    v.pass.push_back(pass);
    return true;
}

bool read_vcf(const std::string& path, const vp_call_filter& cf, Vcf& v) {
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
        if (cols.size() < 9 || !line_info(line.data(), line.data() + line.size(), v)) return false;
        int nalt = 1;
        for (char ch : cols[4]) nalt += ch == ',';
        v.k.push_back(1 + nalt);
        // FORMAT keys of the genotype filter, and each call's offset in the line
        int dpid = -1, gqid = -1;
        uint64_t kept = 0;
        vp::parse_format(cols[8].data(), (int64_t)cols[8].size(), &dpid, &gqid, &kept);
        std::vector<size_t> at(cols.size());
        for (size_t c = 1, off = 0; c < cols.size(); ++c) { off += cols[c - 1].size() + 1; at[c] = off; }
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
            if (vp::call_filtered(cf, line.data(), (int64_t)at[9 + i], (int64_t)line.size(), dpid, gqid, kept, n)) continue;
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
    if (vp_vcf_pack2_ex(data, bytes, N, o.device, packed.data(), L, starts.data(), &got, &o.cf) || got != L) {
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
        if (vp_vcf_parse_ex(data, bytes, N, vmax, o.device, v.G.data(), v.k.data(), v.ploidy.data(), L,
                            starts.data(), &got, &o.cf) || got != L) {
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
            if (!t1 || !t2 || !t3 || !line_info(a, e, v)) { v = Vcf(); return 0; }
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
        if (!t1 || !t2 || !t3 || !line_info(a, e, v)) { v = Vcf(); packed.clear(); return 0; }
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
bool individual_filter(const Opts& o, Vcf& v, bool dev_ingest, std::vector<uint32_t>& packed, std::vector<int>& pop,
                       std::vector<int>& kept) {
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
    kept = keep;
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

// The loader's locus tests on the fixed columns (LOCUS::LOCUS, src/function.cpp
// :3258-3290): -f_type=snp drops indels and =indel drops the other loci;
// -f_original=yes drops loci whose FILTER does not start with "pass";
// -f_chrprefix keeps chromosomes that start with one of its prefixes (LineCmp,
// src/string2.cpp:222-231), -f_chrname those equal to one of its names.
void info_filter(const Opts& o, const Vcf& v, std::vector<uint8_t>& keep) {
    for (size_t l = 0; l < keep.size(); ++l) {
        bool pass = keep[l];
        if (pass && o.type_val == 1 && v.indel[l]) pass = false;
        if (pass && o.type_val == 2 && !v.indel[l]) pass = false;
        if (pass && o.original_b && !v.pass[l]) pass = false;
        if (pass && o.chrprefix_b) {
            pass = false;
            for (const auto& pr : o.chrprefix) pass |= v.chrom[l].compare(0, pr.size(), pr) == 0 && v.chrom[l].size() >= pr.size();
        }
        if (pass && o.chrname_b) {
            pass = false;
            for (const auto& nm : o.chrname) pass |= v.chrom[l] == nm;
        }
        keep[l] = pass;
    }
}

// The window filter (MarkerDiversity, src/filter.cpp:509-555, then 74-90):
// of the loci that pass, each window (CHROM, (POS - 1) / -f_windowsize)
// keeps one, the first in file order with the largest -f_windowstat
// statistic (a later locus replaces it only with a strictly larger value:
// the reference's order with one thread); every other locus fails. st holds
// the device statistics, VP_LOCUS_STATS per locus.
void window_filter(const Opts& o, const Vcf& v, const std::vector<double>& st, std::vector<uint8_t>& keep) {
    // -f_windowstat 1..8 (bmaf, k, n, ptype, he, ho, pic, ae) -> statistic column (n, k, ptype, bmaf, he, ho, pic, ae, ...)
    static const int col[9] = {4, 3, 1, 0, 2, 4, 5, 6, 7};
    const int c = col[o.windowstat];
    std::map<std::pair<std::string, int64_t>, std::pair<int64_t, double>> best;
    for (size_t l = 0; l < keep.size(); ++l) {
        if (!keep[l]) continue;
        const double div = st[l * VP_LOCUS_STATS + c];
        const auto key = std::make_pair(v.chrom[l], (v.pos[l] - 1) / o.windowsize);
        auto it = best.find(key);
        if (it == best.end()) best.emplace(key, std::make_pair((int64_t)l, div));
        else if (it->second.second < div) it->second = std::make_pair((int64_t)l, div);
    }
    std::fill(keep.begin(), keep.end(), 0);
    for (const auto& w : best) keep[w.second.first] = 1;
}

}  // namespace

int main(int argc, char** argv) {
    Opts o;
    if (!parse(argc, argv, o)) return 2;
    Vcf v;
    std::vector<uint32_t> dev_packed;   // device-parsed 2-bit matrix, file order of individuals
    const int ingest = read_vcf_device(o, v, dev_packed);
    const bool dev_ingest = ingest == 1;   // the 2-bit matrix (else allele copies in v.G)
    if (!ingest && !read_vcf(o.input, o.cf, v)) { fprintf(stderr, "vcfpop-gb300: cannot read %s\n", o.input.c_str()); return 2; }
    const int N0 = (int)v.inds.size();
    const int64_t L0 = (int64_t)v.k.size();
    // with the genotype filter, the loader's genotype table still holds
    // every call of the file (src/load.cpp:2145-2230): which loci are
    // polymorphic and how the loci are ordered follow the calls before the
    // filter, read here a second time without it
    std::vector<uint8_t> tpoly;
    std::vector<int32_t> tngeno;
    Vcf v0;    // the calls before the genotype filter, file order (general layout)
    if (o.filter && (o.cf.dp_b || o.cf.gq_b || o.cf.ploidy_b)) {
        Opts o0 = o;
        o0.cf = vp_call_filter{};
        std::vector<uint32_t> p0;
        const int k0 = read_vcf_device(o0, v0, p0);
        if (!k0 && !read_vcf(o.input, o0.cf, v0)) { fprintf(stderr, "vcfpop-gb300: cannot read %s\n", o.input.c_str()); return 2; }
        if ((int64_t)v0.k.size() != L0 || (int)v0.inds.size() != N0) { fprintf(stderr, "vcfpop-gb300: the second read differs\n"); return 1; }
        vp_input t{};
        t.n_ind = N0; t.n_loc = L0; t.vmax = v0.vmax; t.ploidy = v0.ploidy.data(); t.n_alleles = v0.k.data();
        if (k0 == 1) t.packed2 = p0.data();
        else t.alleles = v0.G.data();
        tpoly.resize(L0);
        tngeno.resize(L0);
        if (vp_genotype_table(&t, tpoly.data(), tngeno.data())) { fprintf(stderr, "vcfpop-gb300: %s\n", vp_last_error()); return 1; }
        if (k0 == 1) v0.G.clear();
    }
    std::vector<int> pop;
    std::vector<std::string> pnames;
    populations(o.indtext, N0, pop, pnames);
    std::vector<int> kept_inds;
    if (o.filter && (o.itype_b || o.iploidy_b)) {
        if (!individual_filter(o, v, dev_ingest, dev_packed, pop, kept_inds)) return 1;
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
    // the locus filters (src/filter.cpp ApplyFilter), over the loci of the
    // file: the loader's tests on the fixed columns (-f_type, -f_original,
    // -f_chrprefix, -f_chrname), then, on the device for the packed matrix,
    // the diversity windows (MarkerDiversity) and the window filter over the
    // loci that passed; the loci that fail are dropped here
    const vp_locus_filter& lf = o.lf;
    const bool windows = lf.bmaf_b || lf.k_b || lf.n_b || lf.ptype_b || lf.he_b || lf.ho_b || lf.pic_b || lf.ae_b ||
                         lf.I_b || lf.pval_b;
    const bool info_tests = o.type_val == 1 || o.type_val == 2 || o.original_b || o.chrprefix_b || o.chrname_b;
    std::vector<uint32_t> kept_packed;
    std::vector<int8_t> kept_G;
    if (o.filter && (windows || info_tests || o.windowsize)) {
        std::vector<uint8_t> keep(L0, 1);
        if (info_tests) info_filter(o, v, keep);
        if (windows || o.windowsize) {
            std::vector<uint8_t> kd(L0);
            std::vector<double> st(o.windowsize ? (size_t)L0 * VP_LOCUS_STATS : 0);
            int frc;
            if (in.packed2) {
                frc = vp_locus_filter_pack2(in.packed2, L0, N, &lf, o.device, kd.data(), o.windowsize ? st.data() : nullptr);
            } else {
                // the general layout, in the file's order of individuals (the
                // order in which the loader met each genotype); with the
                // genotype filter, the calls before it order the tables
                int maxp = 0;
                for (int i = 0; i < N; ++i) maxp = std::max(maxp, (int)v.ploidy[i]);
                if (lf.pval_b && o.model_val && maxp >= 4) {
                    fprintf(stderr, "vcfpop-gb300: -f_model with -f_pval on data of ploidy 4 or more is not implemented "
                                    "(the double-reduction genotype frequencies)\n");
                    return 1;
                }
                std::vector<int8_t> tsub;
                const int8_t* table = nullptr;
                if (!v0.G.empty()) {
                    if (kept_inds.empty()) table = v0.G.data();
                    else {
                        tsub.resize(v.G.size());
                        for (int64_t l = 0; l < L0; ++l)
                            for (size_t j = 0; j < kept_inds.size(); ++j)
                                memcpy(&tsub[((size_t)l * N + j) * v.vmax], &v0.G[((size_t)l * N0 + kept_inds[j]) * v.vmax],
                                       v.vmax);
                        table = tsub.data();
                    }
                }
                frc = vp_locus_filter_general(v.G.data(), table, L0, N, v.vmax, v.k.data(), &lf, o.device, kd.data(),
                                              o.windowsize ? st.data() : nullptr);
            }
            if (frc) {
                fprintf(stderr, "vcfpop-gb300: %s\n", vp_last_error());
                return 1;
            }
            for (int64_t l = 0; l < L0; ++l) keep[l] &= kd[l];
            if (o.windowsize) window_filter(o, v, st, keep);
        }
        int64_t nk = 0;
        for (int64_t l = 0; l < L0; ++l) nk += keep[l];
        if (nk == 0) { fprintf(stderr, "vcfpop-gb300: all %lld loci are excluded by the filters\n", (long long)L0); return 1; }
        std::vector<int32_t> k2;
        std::vector<std::string> locs2;
        if (in.packed2) {
            const int Nw = (N + 15) / 16;
            kept_packed.resize((size_t)nk * Nw);
            for (int64_t l = 0, j = 0; l < L0; ++l)
                if (keep[l]) memcpy(&kept_packed[(size_t)j++ * Nw], in.packed2 + (size_t)l * Nw, (size_t)Nw * 4);
            in.packed2 = kept_packed.data();
        } else {
            const size_t row = (size_t)N * v.vmax;
            kept_G.resize((size_t)nk * row);
            for (int64_t l = 0, j = 0; l < L0; ++l)
                if (keep[l]) memcpy(&kept_G[(size_t)j++ * row], in.alleles + (size_t)l * row, row);
            in.alleles = kept_G.data();
        }
        for (int64_t l = 0, j = 0; l < L0; ++l)
            if (keep[l]) {
                k2.push_back(v.k[l]);
                locs2.push_back(v.locs[l]);
                if (!tpoly.empty()) { tpoly[j] = tpoly[l]; tngeno[j] = tngeno[l]; ++j; }
            }
        v.k.swap(k2);
        v.locs.swap(locs2);
        in.n_loc = nk;
        in.n_alleles = v.k.data();
        fprintf(stderr, "vcfpop-gb300: locus filters kept %lld of %lld loci\n", (long long)nk, (long long)L0);
    }
    if (!tpoly.empty()) { in.table_poly = tpoly.data(); in.table_ngeno = tngeno.data(); }
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
