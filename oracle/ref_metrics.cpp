// The reference's own metric evaluators (shared/metric.cpp), compiled as they are
// into oracle/_ref/libref_metrics.so -- TEST INFRASTRUCTURE ONLY.  They read a
// refinement state in the reference's layout (ep_starts, ep_ends = lambda(e),
// ep_parts, ep_cnt), so handing them a state that the engine wrote
// (fp_get_state, fp_stream_partition) checks that the layout is the
// reference's: the values must equal the engine's own metrics.
//
// ref_metrics(): the six values in the reference's print order (TV, CN, TM,
// MGM, MGV, MGAV) as partition_gpu() evaluates them after refinement
// (TV/partition.cpp:1126-1131): TV_Refined over ep_starts / ep_cnt, CN over
// ep_ends, TM_scratch, MGM_scratch, MGV_Scratch and MGAV_Scratch over the
// vertex -> nets CSR with true net sizes.  out[6] also gets TV(ep_ends) in
// out[6], the form partition_gpu() prints before refinement.
#include <vector>
#include "metric.h"

extern "C" int ref_metrics(int K, int nov, int noe, long long pins, const unsigned* row_ptr,
                           const unsigned* col_ind, const unsigned* net_sizes, const int* src_nodes,
                           const int* part_vec, const int* ep_starts, const int* ep_ends, const int* ep_parts,
                           const int* ep_cnt, long long* out) {
  // The evaluators take non-const pointers and TV_Refined reads ep_starts[noe].
  std::vector<unsigned> rp(row_ptr, row_ptr + nov + 1), ci(col_ind, col_ind + pins), ns(net_sizes, net_sizes + noe);
  std::vector<int> src(src_nodes, src_nodes + noe), pv(part_vec, part_vec + nov);
  std::vector<int> st(ep_starts, ep_starts + noe), en(ep_ends, ep_ends + noe);
  std::vector<int> pa(ep_parts, ep_parts + pins), cn(ep_cnt, ep_cnt + pins);
  st.push_back((int)pins);
  out[0] = TV_Refined(st.data(), cn.data(), noe, K);
  out[1] = CN(en.data(), noe);
  out[2] = TM_scratch(K, pv.data(), pa.data(), st.data(), en.data(), nov, noe, src.data());
  out[3] = MGM_scratch(K, pv.data(), pa.data(), st.data(), en.data(), nov, noe, src.data());
  out[4] = MGV_Scratch(pv.data(), rp.data(), ci.data(), src.data(), en.data(), ns.data(), K, nov, noe, (int)pins);
  out[5] = MGAV_Scratch(pv.data(), rp.data(), ci.data(), src.data(), en.data(), pa.data(), st.data(), ns.data(), K,
                        nov, noe, (int)pins);
  out[6] = TV(en.data(), noe);
  return 0;
}
