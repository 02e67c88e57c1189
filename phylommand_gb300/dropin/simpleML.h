/* Drop-in replacement of phylommand's simpleML (src/simpleML.h:30-142) that
 * computes on a GB300 through libplk (include/plk.h).
 *
 * Same class name, base class and public methods as the reference, so
 * treeator.cpp compiles and links unchanged: put this directory before the
 * reference's src/ on the include path, compile simpleML.cpp from here
 * instead of the reference's, and link libplk.so.
 *
 *   reference                                   here
 *   set_char            (src/simpleML.h:41-57)  stores the state set per site
 *   calculate_log_likelihood (src/simpleML.h:58-90, src/simpleML.cpp:127-197)
 *                                               flattens the tree, plk_loglik
 *   calculate_likelihood_rate_change_at_nodes / _in_time (src/simpleML.h:75, 91)
 *                                               same, with the rate_model's
 *                                               time slices and clade rates
 *   draw_normalized_likelihood_on_nodes (src/simpleML.cpp:199-231)
 *                                               plk_node_states, same label text
 *   simulate_chars      (src/simpleML.cpp:233-292)  host, rand() as the reference
 *   get_n_char          (src/simpleML.cpp:41-50)
 *
 * Environment: PLK_DEVICE (default 0); PLK_PRECISION=fp32s selects the FP32
 * scaled form (default FP64, the reference's operation order).  Failures
 * print to cerr and return 0.0, as the reference does for bad tip data.
 */
#ifndef SIMPLEML_GPU_DROPIN_H
#define SIMPLEML_GPU_DROPIN_H

#include <bitset>
#include <cmath>
#include <iostream>
#include <map>
#include <vector>

#include "partition_models.h"
#include "plk.h"
#include "sub_model.h"
#include "tree.h"

using namespace std;

class simpleML : public tree {
  public:
    simpleML() : plk_(0), data_dirty_(true) {}
    ~simpleML();
    void init() { tips_.clear(); data_dirty_ = true; }
    void reset() { init(); }
    void set_char(const int char_no, const string taxon, const bitset<SIZE>& state, sub_model& model);
    double calculate_log_likelihood(sub_model& model) {
        rate_model rate_mod;
        return calculate_log_likelihood(model, rate_mod);
    }
    double calculate_likelihood_rate_change_at_nodes(rate_model& rate_mod, sub_model& model) {
        return calculate_log_likelihood(model, rate_mod);
    }
    double calculate_log_likelihood(sub_model& model, rate_model& rate_mod);
    double calculate_likelihood_rate_change_in_time(rate_model& rate_mod, sub_model& model) {
        return calculate_log_likelihood(model, rate_mod);
    }
    vector<character_vector> simulate_chars(const vector<double>& charfreq, const unsigned int n_char,
                                            sub_model& model);
    void draw_normalized_likelihood_on_nodes();
    unsigned int get_n_char(node* leaf);

  private:
    // state sets per tip and site, as set_char received them
    map<node*, vector<bitset<SIZE> > > tips_;
    plk_handle* plk_;
    bool data_dirty_;
    // flattened tree of the last upload
    vector<node*> nodes_;         // id -> node (tips first)
    vector<int> left_, right_;
    vector<double> bl_;
    unsigned int n_states_uploaded_ = 0;
    int precision() const;
    bool ensure_handle();
    bool flatten(vector<node*>* nodes, vector<int>* left, vector<int>* right, vector<double>* bl);
    bool upload(sub_model& model, rate_model& rate_mod);
    void simulate_subtree(node* leaf, map<node*, unsigned int>& sim, unsigned int ancestor, sub_model& model);
};

#endif
