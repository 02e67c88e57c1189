// Test infrastructure (oracle side): a command-line driver around the
// reference's own simpleML / sub_model / rate_model objects, compiled from the
// reference sources where they lie (oracle/Makefile).  Only tests and the
// CPU-baseline leg of bench.py use it, as a checker; the product never links it.
//
// What it does, and which reference behaviour it follows:
//  * reads a FASTA alignment with the reference's matrix_parser and alphabet
//    (DNA built in, or an alphabet file), then sets empty cells to "all
//    states" as treeator does (src/treeator.cpp:463-466);
//  * parses the Newick tree with tree::tree_file_parser (src/tree.cpp:69-237);
//  * sets EVERY site with simpleML::set_char (src/simpleML.h:41-57), where the
//    treeator CLI sets only site 0 (src/treeator.cpp:723-724);
//  * builds the sub_model without calling set_rate_spec for more than one
//    distinct rate (its allocation at src/sub_model.cpp:87 holds one double),
//    writing rate_specs / rates / state_freqs through the opened-up class and
//    then calling set_rate so that calc_Q_matrix runs with the final values
//    (src/sub_model.cpp:99-114).  No arithmetic of the reference is changed;
//  * runs calculate_log_likelihood (src/simpleML.h:76-90) unchanged, or, with
//    --no-root-quirk, the same private recursion started at a root distance
//    of 1e-30 instead of 0, so that rate_model::get_time_mod_branch_length
//    (src/rate_model.cpp:103-127) returns the raw branch length for the two
//    root-child edges;
//  * for K rate categories (absent in the reference) runs K passes with every
//    node::branchlength multiplied by r_k in double and mixes the per-site
//    root sums with weights w_k in the harness.
//
// Output (stdout, %.17g):
//   T <postorder_id> <is_tip> <left_id> <right_id> <branchlength> <label>
//   C <postorder_id> <clade_no>   (MRCA nodes of --clade-rates taxon sets)
//   S <site> <site_loglik>
//   L <total_loglik>
//   N <internal_postorder_rank> <cat> <site> <v_0> ... <v_{S-1}>   (raw cond.)
//   Q <row> <q_i0> ... (the reference's Q matrix)
//   P <t> <row> <p_i0> ... (sub_model::set_P_matrix(t) for each --pmat t)
//   TIME <seconds per evaluation>
//   D <row> <taxon> <mask_0,mask_1,...> (hex state sets, with --dump-tips)
// --nsites K scores only the first K sites (the CLI itself scores site 0).
// --time-rates / --clade-rates take treeator's -U and -V argument strings.
#include <iostream>
#include <sstream>
#include <fstream>
#include <map>
#include <vector>
#include <set>
#include <string>
#include <bitset>
#include <forward_list>
#include <algorithm>
#include <cmath>
#include <limits>
#include <ctime>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#define private public
#define protected public
#include "simpleML.h"
#undef private
#undef protected

typedef tree::node rnode;

static std::vector<double> parse_list(const char* s) {
    std::vector<double> out;
    std::string cur;
    for (const char* p = s;; ++p) {
        if (*p == ',' || *p == '\0') {
            if (!cur.empty()) out.push_back(atof(cur.c_str()));
            cur.clear();
            if (*p == '\0') break;
        } else cur += *p;
    }
    return out;
}

static void postorder(rnode* n, std::vector<rnode*>& out) {
    if (n == 0) return;
    postorder(n->left, out);
    postorder(n->right, out);
    out.push_back(n);
}

static void scale_bl(rnode* n, double f, std::map<rnode*, double>& orig) {
    if (n == 0) return;
    orig[n] = n->branchlength;
    n->branchlength = n->branchlength * f;
    scale_bl(n->left, f, orig);
    scale_bl(n->right, f, orig);
}

int main(int argc, char** argv) {
    std::string fasta, treefile, alphabet_file;
    std::vector<double> rates, specs, freqs, gamma_r, gamma_w, pmats;
    bool tr = false, have_freqs = false, quirk = true, nodes = false, sites = false;
    int repeat = 0;
    long max_sites = -1;
    bool dump_tips = false;
    std::string time_rates_arg, clade_rates_arg;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        if (a == "--fasta") fasta = argv[++i];
        else if (a == "--tree") treefile = argv[++i];
        else if (a == "--alphabet") alphabet_file = argv[++i];
        else if (a == "--rates") rates = parse_list(argv[++i]);
        else if (a == "--specs") specs = parse_list(argv[++i]);
        else if (a == "--freqs") { freqs = parse_list(argv[++i]); have_freqs = true; }
        else if (a == "--tr") tr = atoi(argv[++i]) != 0;
        else if (a == "--cat-rates") gamma_r = parse_list(argv[++i]);
        else if (a == "--cat-weights") gamma_w = parse_list(argv[++i]);
        else if (a == "--no-root-quirk") quirk = false;
        else if (a == "--nodes") nodes = true;
        else if (a == "--sites") sites = true;
        else if (a == "--pmat") pmats = parse_list(argv[++i]);
        else if (a == "--time") repeat = atoi(argv[++i]);
        else if (a == "--nsites") max_sites = atol(argv[++i]);
        else if (a == "--dump-tips") dump_tips = true;
        else if (a == "--time-rates") time_rates_arg = argv[++i];
        else if (a == "--clade-rates") clade_rates_arg = argv[++i];
        else { std::cerr << "unknown argument " << a << std::endl; return 2; }
    }
    if (have_freqs) tr = true;  // as treeator does (src/treeator.cpp:553)
    // alphabet (src/treeator.cpp:396-421)
    std::map<char, std::bitset<SIZE> > alphabet;
    if (alphabet_file.empty() || alphabet_file == "dna") alphabet::set_alphabet_dna(alphabet);
    else {
        std::ifstream af(alphabet_file.c_str());
        alphabet_parser parser(af, alphabet);
        parser.pars();
    }
    std::bitset<SIZE> all_possible;
    for (std::map<char, std::bitset<SIZE> >::const_iterator i = alphabet.begin(); i != alphabet.end(); ++i)
        all_possible |= i->second;
    partitions regions;
    regions.add_alphabet("first", alphabet);
    regions.add_partition(0, 0, "default", "first");
    std::vector<character_vector> characters;
    {
        std::ifstream df(fasta.c_str());
        if (!df.good()) { std::cerr << "cannot open " << fasta << std::endl; return 2; }
        matrix_parser data_parser(df, characters, regions, "fasta");
        data_parser.pars();
    }
    for (size_t i = 0; i < characters.size(); ++i) characters[i].set_empty_to(all_possible);
    unsigned int n_states = 0;
    for (size_t i = 0; i < characters.size(); ++i)
        if (characters[i].highest_char_state() + 1 > n_states) n_states = characters[i].highest_char_state() + 1;
    unsigned int n_char = characters.empty() ? 0 : characters[0].n_char();
    if (max_sites >= 0 && (unsigned long)max_sites < n_char) n_char = (unsigned int)max_sites;
    if (dump_tips)
        for (size_t i = 0; i < characters.size(); ++i) {
            printf("D %zu %s", i, characters[i].get_taxon().c_str());
            for (unsigned int s = 0; s < n_char; ++s)
                printf("%c%lx", s ? ',' : ' ', characters[i].get_character(s).to_ulong());
            printf("\n");
        }

    // model
    sub_model model(n_states, tr);
    unsigned int npos = model.n_posible_rates();
    unsigned int max_spec = 0;
    for (unsigned int i = 0; i < npos; ++i) {
        unsigned int s = i < specs.size() ? (unsigned int)specs[i] : 0;
        model.rate_specs[i] = s;
        if (s > max_spec) max_spec = s;
    }
    delete[] model.rates;
    model.rates = new double[max_spec + 1];
    model.n_rates = max_spec + 1;
    for (unsigned int i = 0; i <= max_spec; ++i) model.rates[i] = 1.0;
    if (tr && model.state_freqs != 0) {
        for (unsigned int i = 0; i < n_states; ++i)
            model.state_freqs[i] = (have_freqs && i < freqs.size()) ? freqs[i] : 1.0 / n_states;
    }
    for (unsigned int i = 0; i <= max_spec; ++i)
        model.set_rate(i, i < rates.size() ? rates[i] : (tr ? 1.0 : 0.1));
    for (unsigned int r = 0; r < n_states; ++r) {
        printf("Q %u", r);
        for (unsigned int c = 0; c < n_states; ++c) printf(" %.17g", model.Q_matrix->get_value(r, c));
        printf("\n");
    }
    for (size_t k = 0; k < pmats.size(); ++k) {
        model.set_P_matrix(pmats[k]);
        for (unsigned int r = 0; r < n_states; ++r) {
            printf("P %.17g %u", pmats[k], r);
            for (unsigned int c = 0; c < n_states; ++c) printf(" %.17g", model.get_P_value(r, c));
            printf("\n");
        }
    }
    if (treefile.empty()) return 0;

    // tree
    simpleML tr_obj;
    {
        std::ifstream tf(treefile.c_str());
        std::map<std::string, std::string> trans;
        tr_obj.tree_file_parser(tf, trans, false);
    }
    // rate model: -U/-S style "rate:cut,..." and -V style "rate:taxA,taxB;..."
    // arguments, parsed by the reference (src/rate_model.cpp:129-175)
    rate_model rate_mod;
    std::vector<std::string> taxon_sets;
    if (!time_rates_arg.empty() && !rate_mod.pars_rates_and_times_arg(time_rates_arg.c_str())) {
        std::cerr << "bad --time-rates" << std::endl; return 2;
    }
    if (!clade_rates_arg.empty() && !rate_mod.pars_clade_rates_arg(clade_rates_arg.c_str(), taxon_sets)) {
        std::cerr << "bad --clade-rates" << std::endl; return 2;
    }
    if (!taxon_sets.empty()) tr_obj.add_taxon_sets(taxon_sets);
    tr_obj.init();
    for (size_t i = 0; i < characters.size(); ++i)
        for (unsigned int s = 0; s < n_char; ++s)
            tr_obj.set_char(s, characters[i].get_taxon(), characters[i].get_character(s), model);

    std::vector<rnode*> po;
    postorder(tr_obj.root, po);
    std::map<rnode*, int> id;
    for (size_t i = 0; i < po.size(); ++i) id[po[i]] = (int)i;
    for (size_t i = 0; i < po.size(); ++i) {
        rnode* n = po[i];
        bool tip = n->left == 0 && n->right == 0;
        printf("T %d %d %d %d %.17g %s\n", (int)i, tip ? 1 : 0, n->left ? id[n->left] : -1,
               n->right ? id[n->right] : -1, n->branchlength,
               (n->nodelabel && !n->nodelabel->empty()) ? n->nodelabel->c_str() : "-");
    }

    for (std::map<rnode*, unsigned int>::iterator it = tr_obj.clades.begin(); it != tr_obj.clades.end(); ++it)
        printf("C %d %u\n", id.count(it->first) ? id[it->first] : -1, it->second);

    if (gamma_r.empty()) { gamma_r.push_back(1.0); gamma_w.push_back(1.0); }
    if (gamma_w.size() != gamma_r.size()) { std::cerr << "cat weights/rates differ in length" << std::endl; return 2; }
    size_t K = gamma_r.size();
    std::vector<double> site_sum;  // per site Σ_k w_k Σ_s L_k[s] π_s
    double t0 = 0.0;
    int reps = repeat > 0 ? repeat : 1;
    std::chrono::steady_clock::time_point start = std::chrono::steady_clock::now();
    for (int rep = 0; rep < reps; ++rep) {
        site_sum.assign(n_char, 0.0);
        for (size_t k = 0; k < K; ++k) {
            std::map<rnode*, double> orig;
            if (!(K == 1 && gamma_r[0] == 1.0)) scale_bl(tr_obj.root, gamma_r[k], orig);
            partition_models models;
            unsigned int nc = tr_obj.get_n_char(tr_obj.root);
            models.add_partition(&model, &rate_mod, 0, nc);
            bool ok = tr_obj.check_nodes(tr_obj.root, models);
            if (!ok) { printf("L 0\n"); return 0; }
            tr_obj.calculate_likelihood(tr_obj.root, models, 0, quirk ? 0.0 : 1e-30);
            std::vector<std::vector<double> >& R = tr_obj.likelihoods[tr_obj.root];
            for (unsigned int pos = 0; pos < R.size() && pos < n_char; ++pos) {
                double lk = 0.0;  // src/simpleML.h:128-135
                for (unsigned int c = 0; c < n_states && c < R[pos].size(); ++c) {
                    if (model.is_tr()) lk += R[pos][c] * model.get_freq(c);
                    else lk += R[pos][c];
                }
                site_sum[pos] += gamma_w[k] * lk;
            }
            if (nodes && rep == 0) {
                int rank = 0;
                for (size_t i = 0; i < po.size(); ++i) {
                    rnode* n = po[i];
                    if (n->left == 0 && n->right == 0) continue;
                    std::vector<std::vector<double> >& V = tr_obj.likelihoods[n];
                    for (unsigned int pos = 0; pos < V.size(); ++pos) {
                        printf("N %d %zu %u", rank, k, pos);
                        for (unsigned int c = 0; c < V[pos].size(); ++c) printf(" %.17g", V[pos][c]);
                        printf("\n");
                    }
                    ++rank;
                }
            }
            for (std::map<rnode*, double>::iterator it = orig.begin(); it != orig.end(); ++it)
                it->first->branchlength = it->second;
        }
    }
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    (void)t0;
    double lnl = 0.0;
    for (unsigned int pos = 0; pos < n_char; ++pos) {
        double ls = log(site_sum[pos]);
        if (sites) printf("S %u %.17g\n", pos, ls);
        lnl += ls;
    }
    printf("L %.17g\n", lnl);
    if (repeat > 0) printf("TIME %.9g\n", secs / reps);
    return 0;
}
