// sodabayes_main.cpp — the `sodabayes` command: the SODABayes job driver
// (SODABayes.f90:1-165, useroptions.f90, the loaders and writers of
// utilities.f90 and models.f90) on top of libsodagpu.so.
//
// It keeps the reference's command line, .par job files (BEGIN name ... END),
// option table and defaults, and writes the same .log/.frq/.hyp/.eff/.mod/.gv
// files in the same formats.  The SODA sampler and the genotype decoding,
// centring and Z build run in the library; this file reads PLINK files,
// parses options and formats output.  Extension: -precision fp64|fp32|fp8
// (default fp64, the reference's arithmetic).  -SODAOff (the regular sampler)
// is not provided: such a job ends with status 1.
#include <sodagpu.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "ffmt.hpp"

using sodahost::Record;

namespace {

struct JobError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// ---- option table (useroptions.f90:18-55) ---------------------------------
enum Kind { K_INT = 1, K_FLOAT = 2, K_CHAR = 3, K_FLAG = 4 };
struct Opt {
    const char *key, *argtype, *desc;
    int kind;
    const char *def;
};
const Opt kOpts[] = {
    {"-parfile", "[filename]", "parameter file", K_CHAR, ""},
    {"-job_name", "[char]", "job name", K_CHAR, ""},
    {"-method", "[char]", "Bayesian method", K_CHAR, "BayesCpi"},
    {"-bfile", "[prefix]", "prefix PLINK binary files", K_CHAR, ""},
    {"-pheno", "[filename]", "alternative phenotype file", K_CHAR, ""},
    {"-pheno_name", "[char]", "phenotype column name", K_CHAR, ""},
    {"-pheno_ncol", "[num]", "phenotype column no.", K_INT, "3"},
    {"-grpfile", "[filename]", "SNP group info file for BayesRc", K_CHAR, ""},
    {"-pi", "[num]", "% SNP with zero effects (BayesB/BayesC)", K_FLOAT, "0.99"},
    {"-scale_va", "[num]", "scale for SNP variance prior", K_FLOAT, "0.01"},
    {"-scale_ve", "[num]", "scale for residual variance prior", K_FLOAT, "0.01"},
    {"-df_va", "[num]", "degrees of freedom Va", K_FLOAT, "0.01"},
    {"-df_ve", "[num]", "degrees of freedom Ve", K_FLOAT, "0.01"},
    {"-alpha", "[num]", "prior for Dirichlet/Beta distribution", K_FLOAT, "1.0"},
    {"-numit", "[num]", "length of MCMC chain", K_INT, "50000"},
    {"-burnin", "[num]", "burnin steps", K_INT, "5000"},
    {"-thin", "[num]", "thinning rate", K_INT, "1"},
    {"-nmix", "[num]", "number of mixture distributions", K_INT, "2"},
    {"-mix", "[num]", "effect sizes of mixtures (% of Va)", K_FLOAT, "0.0,1.0"},
    {"-seed", "[num]", "seed value for random number generator", K_INT, "0"},
    {"-SODAOn", "[flag]", "turn soda on", K_FLAG, "t"},
    {"-SODAOff", "[flag]", "turn soda off", K_FLAG, "f"},
    {"-nthreads", "[num]", "number of threads", K_INT, "1"},
    {"-blocksize", "[num]", "number of SNPs in a block", K_INT, "0"},
    {"-nblocks", "[num]", "number of blocks", K_INT, "0"},
    {"-rblocks", "[flag]", "randomly assign SNPs into blocks", K_FLAG, "f"},
    {"-predict", "[flag]", "perform prediction", K_FLAG, "f"},
    {"-model", "[filename]", "model summary file (for prediction) ", K_CHAR, ""},
    {"-freq", "[filename]", "SNP frequency file (for prediction)", K_CHAR, ""},
    {"-effects", "[filename]", "SNP effect file (for prediction)", K_CHAR, ""},
    {"-out", "[prefix]", "prefix for output", K_CHAR, ""},
    {"-precision", "[char]", "GPU arithmetic: fp64, fp32 or fp8", K_CHAR, "fp64"},
};
const int kNopt = (int)(sizeof kOpts / sizeof kOpts[0]);

std::string upper(std::string s)
{
    for (auto &ch : s) ch = (char)std::toupper((unsigned char)ch);
    return s;
}

bool ssmatch(const std::string &a, const std::string &b) { return upper(a) == upper(b); }

std::string trim(const std::string &s)
{
    size_t b = s.find_first_not_of(" \t\r\n"), e = s.find_last_not_of(" \t\r\n");
    return b == std::string::npos ? std::string() : s.substr(b, e - b + 1);
}

// list-directed style split: blanks, tabs and commas separate items
std::vector<std::string> items(const std::string &line, const char *seps = " \t,")
{
    std::vector<std::string> out;
    std::string cur;
    for (char ch : line) {
        if (std::strchr(seps, ch)) {
            if (!cur.empty()) out.push_back(cur), cur.clear();
        } else {
            cur.push_back(ch);
        }
    }
    if (!cur.empty()) out.push_back(cur);
    return out;
}

// is_key (utilities.f90:179-188): "-" followed by a non-digit
bool is_key(const std::string &s) { return s.size() >= 1 && s[0] == '-' && !(s.size() >= 2 && std::isdigit((unsigned char)s[1])); }

struct Options {
    std::map<std::string, std::string> v;   // key -> value
    Options()
    {
        for (int k = 0; k < kNopt; ++k) v[kOpts[k].key] = kOpts[k].def;
    }
    const std::string &operator[](const std::string &k) const { return v.at(k); }
    bool flag(const std::string &k) const { return v.at(k) == "t"; }
    // parse_parfile_options / parse_cmdline (useroptions.f90:94-205)
    void apply(const std::vector<std::string> &args, const char *where)
    {
        size_t i = 0;
        while (i < args.size()) {
            const std::string &key = args[i];
            if (key.size() > 4 && key.compare(key.size() - 4, 4, ".par") == 0) {
                ++i;
                continue;
            }
            const Opt *o = nullptr;
            for (int k = 0; k < kNopt; ++k)
                if (key == kOpts[k].key) o = &kOpts[k];
            if (!o) throw JobError(std::string("Unknown command line option : ") + key + " (" + where + ")");
            if (o->kind == K_FLAG) {
                v[o->key] = "t";
                ++i;
            } else if (i + 1 >= args.size() || is_key(args[i + 1])) {
                throw JobError(std::string("Missing argument for :") + key + " (" + where + ")");
            } else {
                v[o->key] = args[i + 1];
                i += 2;
            }
        }
    }
};

void show_options()
{
    std::printf("%s\n", "argument    type        description                                default");
    for (int k = 0; k < kNopt; ++k)
        std::printf("%s\n", Record()
                                .a(kOpts[k].key, 12, (int)std::strlen(kOpts[k].key) > 12 ? -1 : 12)
                                .a(kOpts[k].argtype, 12, 12)
                                .a(kOpts[k].desc, 45, 45)
                                .a(kOpts[k].def, 25, 25)
                                .str()
                                .c_str());
}

// cast_float: a default REAL read, i.e. rounded to float32
double cast_float(const std::string &s) { return (double)(float)std::strtod(s.c_str(), nullptr); }
long long cast_int(const std::string &s) { return std::strtoll(s.c_str(), nullptr, 10); }

// ---- job context ------------------------------------------------------------
struct Job {
    std::string name;
    Options opt;
    // files
    std::string inprefix, outprefix, logfil, freqfil, mbvfil, hypfil, modfil, efffil, bedfil, bimfil, famfil;
    bool mcmc = true;
    // data
    int nind = 0, nloci = 0, ngroup = 1;
    std::vector<std::string> animalID, snpID, grpnames;
    std::vector<int32_t> grp;
    std::vector<double> why, freq;
    std::vector<uint8_t> bed;   // payload without the magic bytes
    // options resolved by parse (useroptions.f90:554-...)
    int method = 4, nmix = 2, nthreads = 1, blocksize = 0, nblocks = 0, blockt = 0;
    long long numit = 50000, burnin = 5000, thin = 1, seed1 = 0;
    double pizero = 0.99, scale_va = 0.01, scale_ve = 0.01, df_va = 0.01, df_ve = 0.01;
    std::vector<double> mix, alpha;
    bool sodaoff = false, rblocks = false, alterpheno = false;
    std::string pheno_name;
    int pheno_ncol = 0;
    int precision = SODAGPU_FP64;
    FILE *log = nullptr;
};

const char *kMethods[] = {"BayesA", "BayesB", "BayesC", "BayesCpi", "BayesR", "BayesRc"};

std::string now_stamp(const char *label)
{
    std::time_t t = std::time(nullptr);
    std::tm tmv{};
    localtime_r(&t, &tmv);
    char d[32];
    std::snprintf(d, sizeof d, "%04d-%02d-%02d %02d:%02d:%02d", tmv.tm_year + 1900, tmv.tm_mon + 1, tmv.tm_mday,
                  tmv.tm_hour, tmv.tm_min, tmv.tm_sec);
    // format 101: (a20,1x,a4,'-',a2,'-',a2,' ',a2,':',a2':',a2)
    return sodahost::fmt_a(label, 20) + " " + d;
}

bool file_exists(const std::string &f)
{
    std::ifstream s(f);
    return s.good();
}

std::vector<std::string> read_lines(const std::string &f)
{
    std::ifstream in(f);
    if (!in) throw JobError("cannot open " + f);
    std::vector<std::string> out;
    std::string line;
    while (std::getline(in, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        out.push_back(line);
    }
    return out;
}

// ---- parse (useroptions.f90:554-...) --------------------------------------
void parse(Job &J)
{
    const Options &o = J.opt;
    // parse_out
    J.outprefix = o["-out"];
    J.logfil = J.outprefix + ".log";
    J.freqfil = J.outprefix + ".frq";
    J.mbvfil = J.outprefix + ".gv";
    J.hypfil = J.outprefix + ".hyp";
    J.modfil = J.outprefix + ".mod";
    J.efffil = J.outprefix + ".eff";
    // parse_plink
    J.inprefix = o["-bfile"];
    J.bedfil = J.inprefix + ".bed";
    J.bimfil = J.inprefix + ".bim";
    J.famfil = J.inprefix + ".fam";
    for (const std::string &f : {J.bedfil, J.bimfil, J.famfil})
        if (!file_exists(f)) throw JobError("plink file " + f + " not found");
    // parse_predict
    J.mcmc = !o.flag("-predict");
    if (!J.mcmc) {
        J.modfil = o["-model"];
        J.freqfil = o["-freq"];
        J.efffil = o["-effects"];
        if (J.modfil.empty()) throw JobError("Error: No model file specified");
        if (J.freqfil.empty()) throw JobError("Error: No SNP frequency file specified");
        if (J.efffil.empty()) throw JobError("Error: No SNP effect file specified");
        for (const std::string &f : {J.modfil, J.freqfil, J.efffil})
            if (!file_exists(f)) throw JobError("file " + f + " not found");
        return;
    }
    // parse_method
    J.method = 0;
    for (int m = 0; m < 6; ++m)
        if (ssmatch(o["-method"], kMethods[m])) J.method = m + 1;
    if (!J.method) throw JobError("error: selecting Bayesian method; supported methods: BayesA, BayesB, BayesC, "
                                  "BayesCpi, BayesR, and BayesRc");
    // parse_nmix (useroptions.f90:375-400)
    J.nmix = (int)cast_int(o["-nmix"]);
    if (J.nmix > SODAGPU_MAXDIST) throw JobError("error: max no. of mixture classes exceeded");
    if (J.method == 1) J.nmix = 1;
    if (J.method == 2 || J.method == 3 || J.method == 4) J.nmix = 2;
    // parse_pi
    J.pizero = cast_float(o["-pi"]);
    if (J.pizero <= 0.0 || J.pizero >= 1.0) throw JobError("Error: pi must be a value between 0 and 1");
    // parse_pheno
    J.alterpheno = !o["-pheno"].empty();
    if (J.alterpheno) {
        if (!file_exists(o["-pheno"])) throw JobError("phenotype file " + o["-pheno"] + " not found");
        J.pheno_name = o["-pheno_name"];
        J.pheno_ncol = (int)cast_int(o["-pheno_ncol"]);
    }
    // parse_snpgrp_file
    if (J.method == 6 && !file_exists(o["-grpfile"])) throw JobError("snp group file " + o["-grpfile"] + " not found");
    // parse_soda
    const int maxthreads = std::max(1, (int)std::thread::hardware_concurrency());
    J.nthreads = std::min((int)cast_int(o["-nthreads"]), maxthreads);
    J.sodaoff = o.flag("-SODAOff");   // -SODAOn comes first in the table, so -SODAOff wins
    J.rblocks = o.flag("-rblocks");
    J.blocksize = (int)cast_int(o["-blocksize"]);
    J.nblocks = (int)cast_int(o["-nblocks"]);
    // parse_priors
    J.scale_va = cast_float(o["-scale_va"]);
    J.scale_ve = cast_float(o["-scale_ve"]);
    J.df_va = cast_float(o["-df_va"]);
    J.df_ve = cast_float(o["-df_ve"]);
    J.mix.assign(J.nmix, 0.0);
    J.alpha.assign(J.nmix, 1.0);
    if (J.method == 3 || J.method == 4) {
        J.mix = {0.0, 1.0};
    } else if (J.method >= 5) {
        const auto it = items(o["-mix"], ",");
        if ((int)it.size() != J.nmix)
            throw JobError("Error: Number of mixtue classes " + std::to_string(J.nmix) + " but " +
                           std::to_string(it.size()) + " effect sizes specified (mix)");
        for (int k = 0; k < J.nmix; ++k) J.mix[k] = cast_float(it[k]);
    }
    if (J.method >= 4) {
        const auto it = items(o["-alpha"], ",");
        if (it.size() == 1) {
            for (auto &a : J.alpha) a = cast_float(it[0]);
        } else if ((int)it.size() != J.nmix) {
            throw JobError("Error: Number of mixtue classes " + std::to_string(J.nmix) + " but " +
                           std::to_string(it.size()) + " prior values for Dirichlet specified (alpha)");
        } else {
            for (int k = 0; k < J.nmix; ++k) J.alpha[k] = cast_float(it[k]);
        }
    }
    // parse_initialise
    J.numit = cast_int(o["-numit"]);
    J.burnin = cast_int(o["-burnin"]);
    J.thin = cast_int(o["-thin"]);
    J.seed1 = cast_int(o["-seed"]);
    // extension
    const std::string p = o["-precision"];
    if (p == "fp64") J.precision = SODAGPU_FP64;
    else if (p == "fp32") J.precision = SODAGPU_FP32;
    else if (p == "fp8") J.precision = SODAGPU_FP8;
    else throw JobError("-precision must be fp64, fp32 or fp8");
}

// ---- loaders ----------------------------------------------------------------
void get_size_and_ids(Job &J)
{
    // .fam: one individual per line (get_size counts readable lines)
    for (const auto &l : read_lines(J.famfil)) {
        const auto f = items(l);
        if (f.empty()) continue;
        J.animalID.push_back(f.size() > 1 ? f[1] : f[0]);
        J.why.push_back(f.size() > 5 ? std::strtod(f[5].c_str(), nullptr) : 0.0);
    }
    J.nind = (int)J.animalID.size();
    for (const auto &l : read_lines(J.bimfil)) {
        const auto f = items(l);
        if (f.empty()) continue;
        J.snpID.push_back(f.size() > 1 ? f[1] : f[0]);
    }
    J.nloci = (int)J.snpID.size();
    if (J.mcmc && J.method == 6) {   // groups in order of first appearance (get_size)
        std::vector<std::string> ids;
        for (const auto &l : read_lines(J.opt["-grpfile"])) {
            const auto f = items(l);
            if (f.size() < 2) continue;
            ids.push_back(f[0]);
            int g = -1;
            for (size_t k = 0; k < J.grpnames.size(); ++k)
                if (J.grpnames[k] == f[1]) g = (int)k;
            if (g < 0) {
                J.grpnames.push_back(f[1]);
                g = (int)J.grpnames.size() - 1;
            }
            J.grp.push_back(g + 1);
        }
        if ((int)J.grp.size() < J.nloci) throw JobError("error: reading grpfile: " + J.opt["-grpfile"]);
        for (int j = 0; j < J.nloci; ++j)
            if (ids[j] != J.snpID[j]) throw JobError("error: SNP IDs in grpfile and bimfile not matching");
        J.grp.resize(J.nloci);
        J.ngroup = (int)J.grpnames.size();
        if (J.ngroup > SODAGPU_MAXGRP) throw JobError("error: max no. of SNP groups exceeded");
    }
}

void load_bed(Job &J)
{
    std::ifstream in(J.bedfil, std::ios::binary);
    std::vector<uint8_t> all((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    if (all.size() < 3 || all[0] != 0x6C || all[1] != 0x1B) throw JobError("Binary genotype file may not be a plink file");
    if (all[2] != 0x01) throw JobError("SNP file should not be in individual mode");
    const size_t rec = (size_t)(J.nind + 3) / 4;
    if (all.size() < 3 + rec * (size_t)J.nloci) throw JobError("plink .bed file is shorter than .bim x .fam");
    J.bed.assign(all.begin() + 3, all.begin() + 3 + rec * (size_t)J.nloci);
}

// alternative phenotype file (load_pheno, utilities.f90:339-397)
void load_alt_pheno(Job &J)
{
    const auto lines = read_lines(J.opt["-pheno"]);
    size_t li = 0;
    int col = J.pheno_ncol;
    if (!J.pheno_name.empty()) {
        std::string h = trim(lines.at(0));
        if (h.empty() || h[0] != '$') throw JobError("error: header line must start with $");
        const auto f = items(h.substr(1));
        col = 0;
        for (size_t j = 0; j < f.size(); ++j)
            if (f[j] == J.pheno_name) {
                col = (int)j + 1;
                break;
            }
        if (col <= 0) throw JobError("error: phenotype column name cannot be found.");
        li = 1;
    }
    if (col <= 0) throw JobError("error: phenotype location is not specified.");
    int i = 0;
    for (; li < lines.size() && i < J.nind; ++li) {
        const std::string s = trim(lines[li]);
        if (s.empty() || s[0] == '$') continue;
        const auto f = items(s);
        if (f.size() > 1 && f[1] != J.animalID[i])
            std::printf("error: animal ID %s in phenotype file does not match %s in the plink file.\n", f[1].c_str(),
                        J.animalID[i].c_str());
        if ((int)f.size() < col) throw JobError("phenotype file: too few fields");
        J.why[i] = std::strtod(f[col - 1].c_str(), nullptr);
        ++i;
    }
    if (i < J.nind) std::printf("error: number of records less than %d\n", J.nind);
}

// ---- writers -----------------------------------------------------------------
void write_frq(const Job &J)
{
    FILE *f = std::fopen(J.freqfil.c_str(), "w");
    if (!f) throw JobError("cannot write " + J.freqfil);
    for (int j = 0; j < J.nloci; ++j)   // (A10,1X,F10.6)
        std::fprintf(f, "%s\n", Record().a(J.snpID[j], 10, 80).x().f(J.freq[j], 10, 6).str().c_str());
    std::fclose(f);
}

void write_gv(const Job &J, const std::vector<double> &pred)
{
    FILE *f = std::fopen(J.mbvfil.c_str(), "w");
    if (!f) throw JobError("cannot write " + J.mbvfil);
    for (int i = 0; i < J.nind; ++i)   // (A20,1x,E15.7)
        std::fprintf(f, "%s\n", Record().a(J.animalID[i], 20, 80).x().e(pred[i], 15, 7).str().c_str());
    std::fclose(f);
}

std::string hyp_header(const Job &J)
{
    Record r;
    if (J.method == 1) {   // (A12,3(1x,A15))
        r.a("Iteration", 12).x().a("mu", 15).x().a("Ve", 15).x().a("Va", 15);
    } else if (J.method == 2) {   // ((A12,1x,A12),4(1x,A15))
        r.a("Iteration", 12).x().a("ModelSize", 12).x().a("mu", 15).x().a("Ve", 15).x().a("Va1", 15).x().a("Va2", 15);
    } else {
        r.a("Iteration", 12).x().a("ModelSize", 12).x().a("mu", 15).x().a("Vara", 15).x().a("Ve", 15);
        if (J.ngroup == 1) {
            for (int k = 1; k <= J.nmix; ++k) r.x().a("N" + std::to_string(k), 12);
            for (int k = 1; k <= J.nmix; ++k) r.x().a("Va" + std::to_string(k), 15);
        }
    }
    return r.str();
}

std::string hyp_row(const Job &J, const sodagpu_trace_row &t)
{
    Record r;
    if (J.method == 1) {   // (I12,3(1x,E15.6)): rep, mu, vare, varindist(1)
        r.i(t.rep, 12).x().e(t.mu, 15, 6).x().e(t.vare, 15, 6).x().e(t.varindist[0], 15, 6);
    } else if (J.method == 2) {   // ((I12,1x,I12),4(1x,E15.6)): rep, included, mu, vare, varindist(1:2)
        r.i(t.rep, 12).x().i(t.included, 12).x().e(t.mu, 15, 6).x().e(t.vare, 15, 6);
        r.x().e(t.varindist[0], 15, 6).x().e(t.varindist[1], 15, 6);
    } else {   // ((I12,1x,I12),3(1x,E15.6)) then 20(1x,I12) and 20(1x,E15.6), both non-advancing
        r.i(t.rep, 12).x().i(t.included, 12).x().e(t.mu, 15, 6).x().e(t.vara, 15, 6).x().e(t.vare, 15, 6);
        if (J.ngroup == 1) {
            for (int k = 0; k < J.nmix; ++k) r.x().i(t.snpindist[k], 12);
            if (J.nmix < 20) r.pending();
            for (int k = 0; k < J.nmix; ++k) r.x().e(t.varindist[k], 15, 6);
            if (J.nmix < 20) r.pending();
        }
    }
    return r.str();
}

void write_eff_mod(const Job &J, const std::vector<double> &gstore, const std::vector<double> &indist,
                   const std::vector<double> &vara_sstore, const double scal[4], const std::vector<double> &snpstore,
                   const std::vector<double> &pstore, const std::vector<double> &varstore)
{
    const int m = J.method, nm = J.nmix, ng = J.ngroup;
    FILE *f = std::fopen(J.efffil.c_str(), "w");
    if (!f) throw JobError("Error opening " + J.efffil);
    Record h;
    h.a("snpID", 10, 10).x().a("snpEffect", 15);
    if (m == 1) {
        h.x().a("snpVariance", 15);
    } else {
        if (m == 2) h.x().a("snpVariance", 15);
        for (int k = 1; k <= nm; ++k) h.x().a("PIP" + std::to_string(k), 15);
    }
    std::fprintf(f, "%s\n", h.str().c_str());
    for (int j = 0; j < J.nloci; ++j) {
        Record r;
        r.a(J.snpID[j], 10, 80).x().e(gstore[j], 15, 6);
        if (m == 1 || m == 2) r.x().e(vara_sstore[j], 15, 6);
        if (m != 1)
            for (int k = 0; k < nm; ++k) r.x().e(indist[(size_t)k * J.nloci + j], 15, 6);
        std::fprintf(f, "%s\n", r.str().c_str());
    }
    std::fclose(f);

    f = std::fopen(J.modfil.c_str(), "w");
    if (!f) throw JobError("Error opening " + J.modfil);
    // 800 format(a,t10,E15.6); 801 format(a,t10,a,t15,E15.6); labels are CHARACTER(15)/(10)
    auto w800 = [&](const std::string &lab, int len, double v) {
        std::fprintf(f, "%s\n", Record().a(lab, len >= 0 ? len : (int)lab.size(), len).t(10).e(v, 15, 6).str().c_str());
    };
    auto w801 = [&](const std::string &ca, const std::string &ci, double v) {
        std::fprintf(f, "%s\n", Record().a(ca, 15, 15).t(10).a(ci, 10, 10).t(15).e(v, 15, 6).str().c_str());
    };
    w800("Mean", -1, scal[0]);
    w800("Ve", -1, scal[1]);
    if (m != 1 && m != 2) w800("Vara", -1, scal[2]);
    if (m != 1) {
        w800("NSNP", -1, scal[3]);
        for (int i = 0; i < ng; ++i)
            for (int j = 0; j < nm; ++j) {
                const std::string ci = "N" + std::to_string(j + 1);
                if (ng == 1) w800(ci, 10, snpstore[(size_t)j * ng + i]);
                else w801("Group " + std::to_string(i + 1), ci, snpstore[(size_t)j * ng + i]);
            }
        if (m != 2 && m != 3)
            for (int i = 0; i < ng; ++i)
                for (int j = 0; j < nm; ++j) {
                    const std::string ci = "P" + std::to_string(j + 1);
                    if (ng == 1) w800(ci, 10, pstore[(size_t)j * ng + i]);
                    else w801("Group " + std::to_string(i + 1), ci, pstore[(size_t)j * ng + i]);
                }
    }
    for (int i = 0; i < ng; ++i)
        for (int j = 0; j < nm; ++j) {
            const std::string ci = m == 1 ? std::string("Va") : "Va" + std::to_string(j + 1);
            if (ng == 1) w800(ci, 10, varstore[(size_t)j * ng + i]);
            else w801("Group " + std::to_string(i + 1), ci, varstore[(size_t)j * ng + i]);
        }
    std::fclose(f);
}

// write_log (utilities.f90:198-254)
void write_log(const Job &J)
{
    FILE *f = J.log;
    auto s902 = [&](const std::string &a, const std::string &v) {
        std::fprintf(f, "%s\n", Record().a(a).t(30).a(": ").a(v).str().c_str());
    };
    auto s903 = [&](const std::string &a, long long v) {
        std::fprintf(f, "%s\n", Record().a(a).t(30).a("= ").i(v, 8).str().c_str());
    };
    if (J.mcmc) {
        s902("Prefix for input files", J.inprefix);
        s903("No. of loci", J.nloci);
        s903("No. of individuals", J.nind);
        if (J.alterpheno) {
            s902("Alternative phenotype file", J.opt["-pheno"]);
            if (!J.pheno_name.empty()) s902("Phenotype name", J.pheno_name);
            else s903("Phenotype colunm", J.pheno_ncol);
        }
        std::fprintf(f, "%s\n", Record().a("Prior Vara(Scale DF)").t(30).a("= ").f(J.scale_va, 10, 6).f(J.df_va, 10, 6).str().c_str());
        std::fprintf(f, "%s\n", Record().a("Prior Vare(Scale DF)").t(30).a("= ").f(J.scale_ve, 10, 6).f(J.df_ve, 10, 6).str().c_str());
        s903("No. of MCMC cycles", J.numit);
        s903("Burnin ", J.burnin);
        s903("Thinning rate", J.thin);
        s902("Bayesian method ", kMethods[J.method - 1]);
        auto s905 = [&](const std::string &a, const std::vector<double> &v) {   // (a,t30,'= ',10f10.5)
            for (size_t k0 = 0; k0 < std::max<size_t>(v.size(), 1); k0 += 10) {
                Record r;
                if (k0 == 0) r.a(a).t(30).a("= ");
                for (size_t k = k0; k < std::min(v.size(), k0 + 10); ++k) r.f(v[k], 10, 5);
                std::fprintf(f, "%s\n", r.str().c_str());
            }
        };
        if (J.method == 2 || J.method == 3) {
            s905("pi (%SNP with zero effects)", {J.pizero});
        } else if (J.method >= 5) {
            s903("No. of mixtures", J.nmix);
            s905("Variance of dist ", J.mix);
            s905("Dirichlet prior", J.alpha);
        }
        if (!J.sodaoff) {   // utilities.f90:225-233
            std::fprintf(f, "%s\n", Record().a("SODA on").t(30).a("= ").l(true).str().c_str());
            s903("No. of threads", J.nthreads);
            s903("No. of blocks", J.nblocks);
            s903("Block size", J.blocksize);
            std::fprintf(f, "%s\n", Record().a("Random blocks").t(30).a("= ").l(J.rblocks).str().c_str());
        } else {
            std::fprintf(f, "%s\n", Record().a("SODA off").t(30).a("= ").l(true).str().c_str());
        }
        std::fprintf(f, "%s\n", Record().a("Seed ").t(30).a("= ").i(J.seed1, 12).str().c_str());
        s902("Prefix for output files", J.outprefix);
    } else {
        s902("Prefix for input files", J.inprefix);
        s903("No. of loci", J.nloci);
        s903("No. of individuals", J.nind);
        s902("model file", J.modfil);
        s902("freq file", J.freqfil);
        s902("effects file", J.efffil);
        s902("Prefix for output files", J.outprefix);
    }
    std::fflush(f);
}

void check(int rc, const char *what)
{
    if (rc != 0) {
        const char *msg = sodagpu_last_error();
        throw JobError(std::string(what) + ": " + sodagpu_errstr(rc) + (msg && *msg ? std::string(" (") + msg + ")" : ""));
    }
}

// host Philox4x32-10 (Salmon et al. 2011), for the -rblocks permutation
void philox(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        c[1] = (uint32_t)p1;
        c[3] = (uint32_t)p0;
        c[0] = n0;
        c[2] = n2;
    }
}

// permutate (utilities.f90:588-607) restated with a counter-based stream:
// Fisher-Yates over the SNP positions keyed by the seed.
std::vector<int32_t> random_blocks(int nloci, uint64_t seed)
{
    std::vector<int32_t> perm(nloci);
    for (int j = 0; j < nloci; ++j) perm[j] = j + 1;
    for (int j = nloci - 1; j > 0; --j) {
        uint32_t c[4] = {0u, (uint32_t)j, 8u /* permutation purpose */, 0u};
        philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
        const uint64_t u = ((uint64_t)c[1] << 32) | c[0];
        const int k = (int)(u % (uint64_t)(j + 1));
        std::swap(perm[j], perm[k]);
    }
    return perm;
}

struct HypSink {
    const Job *J;
    FILE *f;
};

void hyp_cb(void *user, const sodagpu_trace_row *row)
{
    HypSink *h = static_cast<HypSink *>(user);
    if (row->chain != 0) return;
    const std::string s = hyp_row(*h->J, *row);
    std::printf("%s\n", s.c_str());
    std::fprintf(h->f, "%s\n", s.c_str());
}

double wall()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// run_program_sodaBayes (SODABayes.f90:112-165)
int run_program(Job &J)
{
    const double t_start = wall();
    parse(J);
    J.log = std::fopen(J.logfil.c_str(), "w");
    if (!J.log) throw JobError("cannot write " + J.logfil);
    std::fprintf(J.log, "Running program SODABayes: %s\n", J.name.c_str());
    std::fprintf(J.log, "%s\n", now_stamp("Run started at").c_str());
    get_size_and_ids(J);
    load_bed(J);
    double t_setup = t_start;
    if (!J.mcmc) {
        // setup_prediction: .frq, .eff, .mod
        J.freq.assign(J.nloci, 0.0);
        const auto fl = read_lines(J.freqfil);
        for (int j = 0; j < J.nloci; ++j) {
            const auto f = items(fl.at(j));
            J.freq[j] = std::strtod(f.at(1).c_str(), nullptr);
        }
        std::vector<double> eff(J.nloci, 0.0);
        const auto el = read_lines(J.efffil);
        for (int j = 0; j < J.nloci; ++j) {
            const auto f = items(el.at(j + 1));
            eff[j] = std::strtod(f.at(1).c_str(), nullptr);
        }
        const auto ml = items(read_lines(J.modfil).at(0));
        const double mu = std::strtod(ml.at(1).c_str(), nullptr);
        std::vector<double> pred(J.nind);
        check(sodagpu_predict(J.nind, J.nloci, J.bed.data(), SODAGPU_GENO_BED, J.freq.data(), mu, eff.data(),
                              pred.data()),
              "sodagpu_predict");
        write_gv(J, pred);
        write_log(J);
    } else {
        if (J.alterpheno) load_alt_pheno(J);
        if (J.seed1 == 0) J.seed1 = (long long)std::chrono::steady_clock::now().time_since_epoch().count() % 2147483647LL;
        int32_t bs = 0, nb = 0, bt = 0;
        // blocksize <= 1 switches SODA off (soda.f90:418-421); -SODAOff runs regular_bayes
        // (SODABayes.f90:136-137)
        if (sodagpu_block_layout(J.nloci, J.nthreads, J.blocksize, J.nblocks, &bs, &nb, &bt) != 0) J.sodaoff = true;
        if (J.sodaoff) {
            bs = J.nloci;
            nb = 1;
            bt = 1;
        }
        J.blocksize = bs;
        J.nblocks = nb;
        J.blockt = bt;
        sodagpu_config cfg{};
        cfg.nind = J.nind;
        cfg.nloci = J.nloci;
        cfg.method = J.method;
        cfg.nmix = J.nmix;
        cfg.ngroup = J.ngroup;
        cfg.blocksize = bs;
        cfg.nblocks = nb;
        cfg.blockt = bt;
        cfg.numit = (int32_t)J.numit;
        cfg.burnin = (int32_t)J.burnin;
        cfg.thin = (int32_t)J.thin;
        cfg.precision = J.precision;
        cfg.sampler = J.sodaoff ? SODAGPU_SAMPLER_REGULAR : SODAGPU_SAMPLER_SODA;
        cfg.chains = 1;
        cfg.recal_every = 1000;
        cfg.seed = std::llabs(J.seed1);
        cfg.pizero = J.pizero;
        cfg.scale_va = J.scale_va;
        cfg.scale_ve = J.scale_ve;
        cfg.df_va = J.df_va;
        cfg.df_ve = J.df_ve;
        for (int k = 0; k < J.nmix; ++k) {
            cfg.mix[k] = J.mix[k];
            cfg.alpha[k] = J.alpha[k];
        }
        sodagpu_ctx *ctx = nullptr;
        check(sodagpu_create(&cfg, &ctx), "sodagpu_create");
        struct Guard {
            sodagpu_ctx *c;
            ~Guard() { sodagpu_destroy(c); }
        } guard{ctx};
        check(sodagpu_load_genotypes(ctx, J.bed.data(), SODAGPU_GENO_BED), "sodagpu_load_genotypes");
        J.freq.assign(J.nloci, 0.0);
        check(sodagpu_get_freq(ctx, J.freq.data()), "sodagpu_get_freq");
        write_frq(J);
        check(sodagpu_load_pheno(ctx, J.why.data()), "sodagpu_load_pheno");
        if (J.method == 6) check(sodagpu_set_groups(ctx, J.grp.data()), "sodagpu_set_groups");
        std::vector<int32_t> perm;
        if (J.rblocks) perm = random_blocks(J.nloci, (uint64_t)std::llabs(J.seed1));
        int32_t nskipped = 0;
        check(sodagpu_build_z(ctx, J.rblocks ? perm.data() : nullptr, &nskipped), "sodagpu_build_z");
        t_setup = wall();
        write_log(J);
        check(sodagpu_init_chains(ctx), "sodagpu_init_chains");
        FILE *hf = std::fopen(J.hypfil.c_str(), "w");
        if (!hf) throw JobError("cannot write " + J.hypfil);
        const std::string head = hyp_header(J);
        std::printf("%s\n", head.c_str());
        std::fprintf(hf, "%s\n", head.c_str());
        HypSink sink{&J, hf};
        const long long chunk = 500;   // rows reach the .hyp file every `chunk` iterations
        for (long long done = 0; done < J.numit; done += chunk) {
            const int it = (int)std::min<long long>(chunk, J.numit - done);
            const int rc = sodagpu_run(ctx, it, hyp_cb, &sink);
            std::fflush(hf);
            if (rc != 0) {
                std::fclose(hf);
                check(rc, "sodagpu_run");
            }
        }
        std::fclose(hf);
        const size_t ngm = (size_t)J.ngroup * J.nmix;
        std::vector<double> gstore(J.nloci), indist((size_t)J.nloci * J.nmix), vss(J.nloci), snp(ngm), pst(ngm),
            var(ngm);
        double scal[4];
        check(sodagpu_get_results(ctx, 0, gstore.data(), indist.data(), vss.data(), scal, snp.data(), pst.data(),
                                  var.data()),
              "sodagpu_get_results");
        write_eff_mod(J, gstore, indist, vss, scal, snp, pst, var);
        std::vector<double> pred(J.nind);
        check(sodagpu_compute_dgv(ctx, scal[0], gstore.data(), pred.data()), "sodagpu_compute_dgv");
        write_gv(J, pred);
    }
    const double t_end = wall();
    std::fprintf(J.log, "%s\n", now_stamp("Run ended at").c_str());
    if (J.mcmc) {
        std::fprintf(J.log, "%s\n", sodahost::fmt_a("Walltime used (seconds)", 31).c_str());
        auto f162 = [](double v) {   // adjustl of an F16.2 field
            std::string s = sodahost::fmt_f(v, 16, 2);
            const size_t b = s.find_first_not_of(' ');
            return s.substr(b) + std::string(b, ' ');
        };
        std::fprintf(J.log, "Setup: %s MCMC: %s Total: %s\n", f162(t_setup - t_start).c_str(),
                     f162(t_end - t_setup).c_str(), f162(t_end - t_start).c_str());
    }
    std::fclose(J.log);
    J.log = nullptr;
    return 0;
}

int run_job(const std::string &name, const std::vector<std::string> &parfile_args,
            const std::vector<std::string> &cmdline)
{
    Job J;
    J.name = name;
    try {
        J.opt.apply(parfile_args, ".par file");
        J.opt.apply(cmdline, "command line");
        if (J.name.empty()) J.name = J.opt["-job_name"];
        std::printf("job %s started...\n", J.name.c_str());
        run_program(J);
    } catch (const std::exception &e) {
        if (J.log) {
            std::fprintf(J.log, "%s\n", e.what());
            std::fclose(J.log);
        }
        std::printf("%s\n", e.what());
        std::printf("job %s did not complete.\n", J.name.c_str());
        return 1;
    }
    std::printf("job %s completed.\n", J.name.c_str());
    return 0;
}

}  // namespace

int main(int argc, char **argv)
{
    std::vector<std::string> cmd(argv + 1, argv + argc);
    if (cmd.empty()) {
        show_options();
        return 0;
    }
    for (const auto &a : cmd)
        if (a.size() >= 2 && a.compare(0, 2, "-h") == 0) {
            show_options();
            return 0;
        }
    if (cmd.size() == 2 && cmd[0] == "--format-selftest") {   // formats one value per descriptor (tests)
        const double v = std::strtod(cmd[1].c_str(), nullptr);
        std::printf("E15.6[%s] E15.7[%s] F10.6[%s] F16.2[%s] I12[%s]\n", sodahost::fmt_e(v, 15, 6).c_str(),
                    sodahost::fmt_e(v, 15, 7).c_str(), sodahost::fmt_f(v, 10, 6).c_str(),
                    sodahost::fmt_f(v, 16, 2).c_str(), sodahost::fmt_i((long long)v, 12).c_str());
        return 0;
    }
    // parse_parfile: -parfile name, or an argument ending in .par
    std::string parfil;
    for (size_t i = 0; i < cmd.size(); ++i) {
        if (cmd[i] == "-parfile" && i + 1 < cmd.size()) {
            parfil = cmd[i + 1];
            break;
        }
        if (cmd[i].size() > 4 && cmd[i].compare(cmd[i].size() - 4, 4, ".par") == 0) {
            parfil = cmd[i];
            break;
        }
    }
    std::vector<std::string> cmdline;
    for (size_t i = 0; i < cmd.size(); ++i) {
        if (cmd[i] == "-parfile") {
            ++i;
            continue;
        }
        cmdline.push_back(cmd[i]);
    }
    if (parfil.empty()) return run_job("", {}, cmdline) ? 1 : 0;
    std::ifstream in(parfil);
    if (!in) {
        std::printf(" par file %s not found\n", parfil.c_str());
        return 1;
    }
    std::string line, job_name;
    std::vector<std::string> params;
    bool in_job = false;
    while (std::getline(in, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        std::string l = trim(line);
        if (l.empty() || l[0] == '#' || l[0] == '!') continue;
        const size_t c = l.find_first_of("#!");
        if (c != std::string::npos) l = trim(l.substr(0, c));
        const auto f = items(l, " \t");
        if (f.empty()) continue;
        if (ssmatch(f[0], "begin")) {
            if (in_job) {
                std::printf(" error: Need an END statement for job: %s\n", job_name.c_str());
                return 1;
            }
            const std::string up = upper(l);
            const size_t p = up.find_first_not_of("BEGIN");
            job_name = p == std::string::npos ? std::string() : trim(l.substr(p));
            params.clear();
            in_job = true;
        } else if (ssmatch(f[0], "end")) {
            if (!in_job) {
                std::printf(" error: need a BEGIN statement to start a job.\n");
                return 1;
            }
            if (run_job(job_name, params, cmdline) != 0) return 1;
            in_job = false;
        } else {
            if (f.size() > 2) {
                std::printf("%s has more than two items\n", l.c_str());
                return 1;
            }
            for (const auto &x : f) params.push_back(x);
        }
    }
    return 0;
}
