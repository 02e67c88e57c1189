// Drop-in simpleML on libplk: see simpleML.h in this directory.
#include "simpleML.h"

#include <cstdlib>
#include <cstring>
#include <sstream>

simpleML::~simpleML() {
    if (plk_) plk_destroy(plk_);
}

int simpleML::precision() const {
    const char* p = getenv("PLK_PRECISION");
    return (p && !strcmp(p, "fp32s")) ? PLK_FP32S : PLK_FP64;
}

bool simpleML::ensure_handle() {
    if (plk_) return true;
    const char* d = getenv("PLK_DEVICE");
    const plk_status s = plk_create(&plk_, d ? atoi(d) : 0);
    if (s != PLK_OK) {
        cerr << "GPU likelihood engine unavailable: " << plk_last_error(0) << endl;
        plk_ = 0;
        return false;
    }
    return true;
}

void simpleML::set_char(const int char_no, const string taxon, const bitset<SIZE>& state, sub_model& model) {
    (void)model;
    node* leaf = find_taxon_tip(root, nodelabels.find_string(taxon));
    if (leaf == 0 || char_no < 0) return;
    vector<bitset<SIZE> >& v = tips_[leaf];
    if ((size_t)char_no >= v.size()) v.resize(char_no + 1);
    v[char_no] = state;
    data_dirty_ = true;
}

// Tips get ids 0..n-1 and internal nodes n.. , both in post-order
// (left subtree, right subtree, node), the order the reference recurses in.
bool simpleML::flatten(vector<node*>* nodes, vector<int>* left, vector<int>* right, vector<double>* bl) {
    vector<node*> post;
    vector<pair<node*, int> > st;
    if (root == 0) return false;
    st.push_back(make_pair(root, 0));
    while (!st.empty()) {
        pair<node*, int>& f = st.back();
        node* u = f.first;
        if (f.second == 0) {
            f.second = 1;
            if (u->left) { st.push_back(make_pair(u->left, 0)); continue; }
        }
        if (f.second == 1) {
            f.second = 2;
            if (u->right) { st.push_back(make_pair(u->right, 0)); continue; }
        }
        post.push_back(u);
        st.pop_back();
    }
    map<node*, int> id;
    nodes->clear();
    for (size_t i = 0; i < post.size(); ++i)
        if (post[i]->left == 0 && post[i]->right == 0) { id[post[i]] = (int)nodes->size(); nodes->push_back(post[i]); }
    for (size_t i = 0; i < post.size(); ++i)
        if (post[i]->left != 0 || post[i]->right != 0) { id[post[i]] = (int)nodes->size(); nodes->push_back(post[i]); }
    const size_t n = nodes->size();
    left->assign(n, -1);
    right->assign(n, -1);
    bl->assign(n, 0.0);
    for (size_t v = 0; v < n; ++v) {
        node* u = (*nodes)[v];
        (*bl)[v] = u->branchlength;
        if (u->left) (*left)[v] = id[u->left];
        if (u->right) (*right)[v] = id[u->right];
    }
    return n >= 2;
}

bool simpleML::upload(sub_model& model, rate_model& rate_mod) {
    if (!ensure_handle()) return false;
    vector<node*> nodes;
    vector<int> left, right;
    vector<double> bl;
    if (!flatten(&nodes, &left, &right, &bl)) {
        cerr << "Tree has no internal node." << endl;
        return false;
    }
    const bool tree_changed = nodes != nodes_ || left != left_ || right != right_ || bl != bl_;
    if (tree_changed) {
        if (plk_set_tree(plk_, (int)nodes.size(), left.data(), right.data(), bl.data()) != PLK_OK) {
            cerr << "GPU likelihood engine: " << plk_last_error(plk_) << endl;
            return false;
        }
        nodes_ = nodes; left_ = left; right_ = right; bl_ = bl;
    }
    const unsigned int S = model.get_n_states();
    if (data_dirty_ || tree_changed || S != n_states_uploaded_) {
        size_t n_tips = 0, n_char = 0;
        for (size_t v = 0; v < nodes.size(); ++v)
            if (nodes[v]->left == 0 && nodes[v]->right == 0) {
                ++n_tips;
                map<node*, vector<bitset<SIZE> > >::const_iterator it = tips_.find(nodes[v]);
                const size_t c = it == tips_.end() ? 0 : it->second.size();
                if (c > n_char) n_char = c;
            }
        vector<uint32_t> masks(n_tips * n_char, 0u);
        for (size_t t = 0; t < n_tips; ++t) {
            map<node*, vector<bitset<SIZE> > >::const_iterator it = tips_.find(nodes[t]);
            if (it == tips_.end() || it->second.size() != n_char) {
                cerr << "Disagreement in number of characters for "
                     << (nodes[t]->nodelabel ? *nodes[t]->nodelabel : string("?")) << endl;
                return false;
            }
            for (size_t s = 0; s < n_char; ++s) masks[t * n_char + s] = (uint32_t)it->second[s].to_ulong();
        }
        if (n_char == 0) {
            cerr << "No characters set." << endl;
            return false;
        }
        if (plk_set_alignment(plk_, (int)n_tips, (int)n_char, (int)S, masks.data()) != PLK_OK) {
            cerr << "GPU likelihood engine: " << plk_last_error(plk_) << endl;
            return false;
        }
        data_dirty_ = false;
        n_states_uploaded_ = S;
    }
    // rate_model through its public getters (src/rate_model.h:50-67)
    vector<float> cut_off(rate_mod.get_n_cut_offs()), cut_rate(rate_mod.get_n_cut_offs());
    for (unsigned int i = 0; i < rate_mod.get_n_cut_offs(); ++i) {
        cut_off[i] = rate_mod.get_cut_off(i);
        cut_rate[i] = rate_mod.get_rate_in_time(i);
    }
    vector<float> clade_rate(rate_mod.get_n_clades());
    for (unsigned int c = 0; c < clade_rate.size(); ++c) clade_rate[c] = rate_mod.get_rate_clade(c);
    vector<int> clade_of_node(nodes.size(), -1);
    bool any_clade = false;
    for (size_t v = 0; v < nodes.size(); ++v) {
        map<node*, unsigned int>::const_iterator it = clades.find(nodes[v]);
        if (it != clades.end() && it->second < clade_rate.size()) {
            clade_of_node[v] = (int)it->second;
            any_clade = true;
        }
    }
    if (plk_set_rate_model(plk_, 1, (int)cut_off.size(), cut_off.empty() ? 0 : cut_off.data(),
                           cut_rate.empty() ? 0 : cut_rate.data(), any_clade ? clade_of_node.data() : 0,
                           (int)clade_rate.size(), clade_rate.empty() ? 0 : clade_rate.data()) != PLK_OK) {
        cerr << "GPU likelihood engine: " << plk_last_error(plk_) << endl;
        return false;
    }
    // Q as sub_model::calc_Q_matrix builds it (src/sub_model.cpp:99-114)
    vector<double> Q(S * S), w(S);
    const bool tr = model.is_tr();
    for (unsigned int i = 0; i < S; ++i) {
        double neg = 0.0;
        for (unsigned int j = 0; j < S; ++j) {
            if (i == j) continue;
            double v = model.get_rate(i, j);
            if (tr) v *= model.get_freq(j);
            neg -= v;
            Q[i * S + j] = v;
        }
        Q[i * S + i] = neg;
        w[i] = tr ? model.get_freq(i) : 1.0;
    }
    const double one = 1.0;
    if (plk_set_model(plk_, (int)S, Q.data(), w.data(), tr ? 1 : 0, 1, &one, &one, PLK_P_TAYLOR20) != PLK_OK) {
        cerr << "GPU likelihood engine: " << plk_last_error(plk_) << endl;
        return false;
    }
    return true;
}

double simpleML::calculate_log_likelihood(sub_model& model, rate_model& rate_mod) {
    if (!upload(model, rate_mod)) return 0.0;
    double lnl = 0.0;
    const plk_status s = plk_loglik(plk_, precision(), &lnl);
    if (s == PLK_ERR_TIP) {
        cerr << "A tip lacks character state for a character!" << endl;
        return 0.0;
    }
    if (s != PLK_OK && s != PLK_ERR_NUMERIC) {
        cerr << "GPU likelihood engine: " << plk_last_error(plk_) << endl;
        return 0.0;
    }
    return lnl;
}

void simpleML::draw_normalized_likelihood_on_nodes() {
    vector<double> out;
    int n_int = 0;
    size_t n_sites = 0;
    unsigned int S = n_states_uploaded_;
    if (plk_ && !nodes_.empty()) {
        n_int = plk_n_internal(plk_);
        for (size_t v = 0; v < nodes_.size(); ++v)
            if (nodes_[v]->left == 0 && nodes_[v]->right == 0) {
                map<node*, vector<bitset<SIZE> > >::const_iterator it = tips_.find(nodes_[v]);
                if (it != tips_.end()) n_sites = it->second.size();
                break;
            }
        out.assign((size_t)n_int * n_sites * S, 0.0);
        if (plk_node_states(plk_, PLK_NODES_COND, precision(), out.data()) != PLK_OK) {
            cerr << "GPU likelihood engine: " << plk_last_error(plk_) << endl;
            n_int = 0;
        }
    }
    // internal nodes of the last upload in post-order rank; label text as
    // src/simpleML.cpp:206-228 writes it
    int rank = 0;
    for (size_t v = 0; v < nodes_.size(); ++v) {
        node* u = nodes_[v];
        if (u->left == 0 && u->right == 0) continue;
        stringstream label;
        label << "[&";
        if (rank < n_int)
            for (size_t site = 0; site < n_sites; ++site) {
                if (site) label << ",";
                label << "P={";
                for (unsigned int s = 0; s < S; ++s) {
                    if (s) label << ',';
                    label << out[((size_t)rank * n_sites + site) * S + s];
                }
                label << "}";
            }
        label << "]";
        string text = label.str();
        if (u->nodelabel != 0) text = *u->nodelabel + text;
        u->nodelabel = nodelabels.add_string(text);
        ++rank;
    }
}

unsigned int simpleML::get_n_char(node* leaf) {
    if (leaf == 0) return 0;
    if (leaf->left == 0 && leaf->right == 0) {
        map<node*, vector<bitset<SIZE> > >::const_iterator it = tips_.find(leaf);
        return it == tips_.end() ? 0 : (unsigned int)it->second.size();
    }
    const unsigned int l = get_n_char(leaf->left), r = get_n_char(leaf->right);
    return l > r ? l : r;
}

// Sequence simulation stays on the host with the C library's rand(), drawing
// in the reference's order: the root state from charfreq, then every node in
// pre-order from the row of P(branch length) of its parent's state.
vector<character_vector> simpleML::simulate_chars(const vector<double>& charfreq, const unsigned int n_char,
                                                  sub_model& model) {
    map<node*, character_vector> by_node;
    for (unsigned int c = 0; c < n_char; ++c) {
        map<node*, unsigned int> sim;
        double u = (double)rand() / RAND_MAX;
        unsigned int root_state = 0;
        for (unsigned int j = 0; j < charfreq.size(); ++j) {
            u -= charfreq[j];
            if (u <= 0) { root_state = j; break; }
        }
        simulate_subtree(root->left, sim, root_state, model);
        simulate_subtree(root->right, sim, root_state, model);
        for (map<node*, unsigned int>::const_iterator it = sim.begin(); it != sim.end(); ++it) {
            bitset<SIZE> b;
            b.set(it->second);
            by_node[it->first].add_character(b);
        }
    }
    vector<character_vector> result;
    for (map<node*, character_vector>::iterator it = by_node.begin(); it != by_node.end(); ++it)
        if (it->first->nodelabel && !it->first->nodelabel->empty()) {
            it->second.set_taxon(*it->first->nodelabel);
            result.push_back(it->second);
        }
    return result;
}

void simpleML::simulate_subtree(node* leaf, map<node*, unsigned int>& sim, unsigned int ancestor, sub_model& model) {
    if (leaf == 0) return;
    model.set_P_matrix(leaf->branchlength);
    unsigned int state = ancestor;
    double u = (double)rand() / RAND_MAX;
    for (unsigned int s = 0; s < model.get_n_states(); ++s) {
        u -= model.get_P_value(ancestor, s);
        if (u <= 0) { state = s; break; }
    }
    sim[leaf] = state;
    simulate_subtree(leaf->left, sim, state, model);
    simulate_subtree(leaf->right, sim, state, model);
}
