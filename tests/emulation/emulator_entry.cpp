
// One engine-mode ant on the host: 32 lane threads run the kernel body of
// variant `mode` (kModeEngine, kModeEngineGlobal, kModeEngineFollow,
// kModeEngineGlobalFollow or kModeEngineFollowDense; the global-workspace
// variants keep the ant's tour and inverse in a host buffer standing for
// the engine's workspace).  Inputs are the instance rows, the colony's
// parent tour with its packed neighbours and products, the Philox key,
// batch and ant index; outputs the ant's final tour, its construction and
// final lengths, and its step / LS / moved counts.  Returns -1 for a mode
// it does not run.
extern "C" int emu_ant(std::uint32_t mode, std::uint32_t n, std::uint32_t k, std::uint32_t b, std::uint32_t w,
                       const int* xy, const std::uint16_t* primary, const std::uint16_t* backup,
                       const std::uint16_t* ls, const int* ls_dist, const std::uint16_t* parent,
                       const std::uint32_t* parent_nbr, const float* products, unsigned long long key,
                       std::uint32_t batch, std::uint32_t ant, std::uint32_t target, long long parent_cost,
                       std::uint32_t ls_mode, std::uint16_t* out_tour, long long* out_costs, unsigned* out_counts,
                       unsigned* error) {
    using namespace faco;
    if (mode != kModeEngine && mode != kModeEngineGlobal && mode != kModeEngineFollow &&
        mode != kModeEngineGlobalFollow && mode != kModeEngineFollowDense)
        return -1;
    const std::uint32_t n_pad = pad8(n);
    InstanceView in{};
    in.n = n; in.k = k; in.b = b; in.w = w;
    in.xy = reinterpret_cast<const int2*>(xy);
    in.primary = primary; in.backup = backup; in.ls = ls; in.ls_dist = ls_dist;
    ColonyView cv{};
    cv.instance = 0; cv.n = n; cv.key = key;
    cv.products = const_cast<float*>(products);
    std::vector<node_t> parent_buf(n_pad + 16, 0);
    node_t* par = parent_buf.data();
    while (reinterpret_cast<std::uintptr_t>(par) & 15) ++par;
    std::memcpy(par, parent, n * sizeof(node_t));
    cv.parent = par;
    cv.parent_nbr = const_cast<std::uint32_t*>(parent_nbr);
    std::vector<node_t> tours_buf(static_cast<std::size_t>(ant + 1) * n_pad + 16, 0);
    node_t* tours = tours_buf.data();
    while (reinterpret_cast<std::uintptr_t>(tours) & 15) ++tours;
    cv.ant_tours = tours; cv.n_pad = n_pad;
    std::vector<long long> costs(ant + 1), ccosts(ant + 1);
    std::vector<unsigned> counts(3 * (ant + 1));
    cv.ant_costs = costs.data(); cv.ant_ccosts = ccosts.data(); cv.ant_counts = counts.data();
    ColonyState st{};
    st.parent_cost = parent_cost; st.mne_target = target; st.iteration = batch; st.region = 4;
    uint2 job{0, ant};
    AntLaunch L{};
    L.instances = &in; L.colonies = &cv; L.states = &st; L.work = &job; L.ants = ant + 1; L.warps = 1;
    L.n_max = n; L.ls_limit = 100000; L.ls_mode = ls_mode; L.error = error;
    // the global-memory workspace: tour and inverse of every ant of the
    // colony, indexed like ant_tours (garbage at first, as on the device)
    std::vector<node_t> workspace(2 * static_cast<std::size_t>(ant + 1) * n_pad + 16, 0xABAB);
    node_t* ws = workspace.data();
    while (reinterpret_cast<std::uintptr_t>(ws) & 15) ++ws;
    L.workspace = ws;
    L.ant_tours_base = tours;
    // shared memory starts with garbage, as on the device
    std::vector<unsigned char> smem(block_smem_bytes(n, 1) + 64, 0xAB);
    unsigned char* sm = smem.data();
    while (reinterpret_cast<std::uintptr_t>(sm) & 15) ++sm;
    Warp warp;
    std::vector<std::thread> th;
    for (unsigned l = 0; l < 32; ++l)
        th.emplace_back([&, l] {
            tl_warp = &warp;
            tl_lane = l;
            switch (mode) {
                case kModeEngine: ant_kernel_emu<kModeEngine>(L, sm); break;
                case kModeEngineGlobal: ant_kernel_emu<kModeEngineGlobal>(L, sm); break;
                case kModeEngineFollow: ant_kernel_emu<kModeEngineFollow>(L, sm); break;
                case kModeEngineGlobalFollow: ant_kernel_emu<kModeEngineGlobalFollow>(L, sm); break;
                case kModeEngineFollowDense: ant_kernel_emu<kModeEngineFollowDense>(L, sm); break;
                default: break;
            }
        });
    for (auto& t : th) t.join();
    std::memcpy(out_tour, tours + static_cast<std::size_t>(ant) * n_pad, n * sizeof(node_t));
    out_costs[0] = ccosts[ant];
    out_costs[1] = costs[ant];
    out_counts[0] = counts[3 * ant];
    out_counts[1] = counts[3 * ant + 1];
    out_counts[2] = counts[3 * ant + 2];
    return 0;
}
