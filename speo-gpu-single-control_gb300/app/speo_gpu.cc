// speo_gpu.cc -- the reference's SPEO_GPU driver (src/main.cc, src/island_EA.cc) on one GPU over
// this library's C ABI.
//
// Same flags as SetParameters (src/main.cc:28-122), same per-run seed (main.cc:138), same FE
// budget loop (island_EA.cc:78-113: RunEA; MigrateOut every `interval` generations from
// generation 0; MigrateIn every generation), same record file ./Results/SPEO_GPU.csv with the
// reference's header (island_EA.cc:13-31) and row (:146-171) and the same console lines. The
// instance is read from ./input_data/ exactly as the reference reads it (M_<f>_D<d>.txt,
// shift_data_<f>.txt, shuffle_data_<f>_D<d>.txt). Differences, by design:
//   * the GPU_num islands (the reference: one MPI rank and GPU each) are an archipelago on this
//     GPU: island i has node_ID i (its seed), its own rows, sub-island permutation, DE parameters
//     and generation counter, and the migration runs through speo_migrate_out / speo_migrate_in
//     (buffer_manage picks the buffer policy: OnlineCluster for "DP" and any other name the
//     reference accepts, which always builds an OnlineCluster; "Best", "Random", "FIFO", "LIFO"
//     select those policies);
//   * FP32 generation (the library's product path), best_fitness re-evaluated in FP64;
//   * -computing_time is accepted and recorded as the reference's app build does (its
//     COMPUTING_TIME switch is off, include/config.h:30): runs stop on the FE budget;
//   * communication_percentage is the share of wall time spent in the migration calls.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "speo_gb300.h"

namespace {

struct Params {
    // ProblemInfo (main.cc:31-37)
    int dim = 100, max_base_FEs = 10000000, computing_time = 10;
    double max_bound = 100, min_bound = -100;
    std::vector<int> functions, runs;
    // NodeInfo / IslandInfo (main.cc:73-90)
    int node_num = 1, GPU_num = 1;
    int island_size = 1024, interval = 10, migration_size = 32, buffer_capacity = 32, subisland_num = 1;
    double migration_rate = 0.5;
    std::string migration_topology = "dynamicConnect", buffer_manage = "DP", regroup_option = "static_and_ordered",
                configure_EA = "constant";
};

const char *get_param(const char *name, int argc, char **argv)
{
    for (int i = 1; i + 1 < argc; ++i)
        if (std::strcmp(argv[i], name) == 0) return argv[i + 1];
    return nullptr;
}

bool parse_range(const char *s, std::vector<int> &out)
{
    int a = 0, b = 0;
    if (!s || std::sscanf(s, "%d-%d", &a, &b) != 2 || b < a) return false;
    out.clear();
    for (int i = a; i <= b; ++i) out.push_back(i);
    return true;
}

int usage(const char *msg)
{
    std::fprintf(stderr, "speo_gpu: %s\n", msg);
    std::fprintf(stderr,
                 "flags (src/main.cc:28-122): -dim D -total_functions a-b -total_runs a-b -computing_time s "
                 "-max_base_FEs n -GPU_num islands -pop_size n -island_size n -interval g -migration_size k "
                 "-migration_topology s -buffer_manage s -regroup_option s -configure_EA constant|dynamic "
                 "-buffer_capacity c -migration_rate p -subisland_size s\n");
    return 2;
}

int set_parameters(Params &p, int argc, char **argv)
{
    for (int i = 23; i <= 30; ++i) p.functions.push_back(i);
    for (int i = 1; i <= 15; ++i) p.runs.push_back(i);
    for (int i = 1; i < argc; i += 2) {
        if (argv[i][0] != '-' || i + 1 >= argc) return usage("flags come as -name value pairs");
    }
    if (const char *v = get_param("-dim", argc, argv)) p.dim = std::atoi(v);
    if (const char *v = get_param("-total_functions", argc, argv))
        if (!parse_range(v, p.functions)) return usage("-total_functions wants a-b");
    if (const char *v = get_param("-total_runs", argc, argv))
        if (!parse_range(v, p.runs)) return usage("-total_runs wants a-b");
    if (const char *v = get_param("-computing_time", argc, argv)) p.computing_time = std::atoi(v);
    if (const char *v = get_param("-max_base_FEs", argc, argv)) p.max_base_FEs = std::atoi(v);
    p.GPU_num = p.node_num;
    if (const char *v = get_param("-GPU_num", argc, argv)) p.GPU_num = std::atoi(v);
    if (const char *v = get_param("-pop_size", argc, argv)) p.island_size = std::atoi(v) / std::max(1, p.GPU_num);
    if (const char *v = get_param("-island_size", argc, argv)) p.island_size = std::atoi(v);
    if (const char *v = get_param("-interval", argc, argv)) p.interval = std::atoi(v);
    if (const char *v = get_param("-migration_size", argc, argv)) p.migration_size = std::atoi(v);
    if (const char *v = get_param("-migration_topology", argc, argv)) p.migration_topology = v;
    if (const char *v = get_param("-buffer_manage", argc, argv)) p.buffer_manage = v;
    if (const char *v = get_param("-regroup_option", argc, argv)) p.regroup_option = v;
    if (const char *v = get_param("-configure_EA", argc, argv)) p.configure_EA = v;
    if (const char *v = get_param("-buffer_capacity", argc, argv)) p.buffer_capacity = std::atoi(v);
    if (const char *v = get_param("-migration_rate", argc, argv)) p.migration_rate = std::atof(v);
    if (const char *v = get_param("-subisland_size", argc, argv)) {
        const int s = std::atoi(v);
        if (s < 1) return usage("-subisland_size must be positive");
        p.subisland_num = p.island_size / s;
    }
    if (p.dim < 1 || p.dim > SPEO_MAX_DIM) return usage("-dim out of range");
    if (p.GPU_num < 1 || p.island_size < 4 || p.interval < 1 || p.max_base_FEs < 1) return usage("bad sizes");
    if (p.subisland_num < 1 || p.island_size % p.subisland_num || p.island_size / p.subisland_num < 4)
        return usage("island_size must split into sub-islands of at least 4 rows (MIN_SUBISLAND_SIZE)");
    if (p.migration_size < 1 || p.migration_size > p.island_size) return usage("bad -migration_size");
    if (p.buffer_capacity < 1 || p.buffer_capacity > SPEO_ARCHIPELAGO_MAX_CAPACITY ||
        p.buffer_capacity > p.island_size)
        return usage("bad -buffer_capacity");
    if (!(p.migration_rate >= 0 && p.migration_rate <= 1)) return usage("bad -migration_rate");
    if (p.configure_EA != "constant" && p.configure_EA != "dynamic") return usage("-configure_EA: constant|dynamic");
    if (p.regroup_option != "static_and_ordered" && p.regroup_option != "static_and_random" &&
        p.regroup_option != "dynamic_and_ordered" && p.regroup_option != "dynamic_and_random")
        return usage("unknown -regroup_option");
    return 0;
}

int buffer_policy(const std::string &s)
{
    if (s == "Best") return SPEO_BUFFER_BEST;
    if (s == "Random") return SPEO_BUFFER_RANDOM;
    if (s == "FIFO") return SPEO_BUFFER_FIFO;
    if (s == "LIFO") return SPEO_BUFFER_LIFO;
    return SPEO_BUFFER_ONLINE_CLUSTER;
}

int regroup_option(const std::string &s)
{
    if (s == "static_and_random") return SPEO_REGROUP_STATIC_RANDOM;
    if (s == "dynamic_and_ordered") return SPEO_REGROUP_DYNAMIC_ORDERED;
    if (s == "dynamic_and_random") return SPEO_REGROUP_DYNAMIC_RANDOM;
    return SPEO_REGROUP_STATIC_ORDERED;
}

int components(int f)
{
    switch (f) {
    case 23: case 26: case 27: case 28: return 5;
    case 24: case 25: case 29: case 30: return 3;
    default: return 1;
    }
}
bool uses_shuffle(int f) { return (f >= 17 && f <= 22) || f == 29 || f == 30; }

std::vector<std::vector<double>> read_lines(const std::string &path, bool &ok)
{
    std::vector<std::vector<double>> out;
    std::ifstream in(path);
    ok = static_cast<bool>(in);
    std::string line;
    while (ok && std::getline(in, line)) {
        std::istringstream ss(line);
        std::vector<double> v;
        double x;
        while (ss >> x) v.push_back(x);
        if (!v.empty()) out.push_back(v);
    }
    return out;
}

// CEC2014_CUDA::LoadData (CUDA_EA_library/CEC2014_CUDA.cc:160-281): shift c at c*np2, M_c^T as np2
// rows of D at c*np2*D (rows >= D zero), shuffle c at c*np2; values as CEC2014::Initilize reads
// them (CEC2014.cc:354-460): M = the first nc*D*D numbers, shift c = the first D numbers of line c
// (the whole file for a single component), shuffle = the first nc*D integers.
bool load_instance(int f, int D, int np2, std::vector<float> &shift, std::vector<float> &rot, std::vector<int> &shuf)
{
    const int nc = components(f);
    bool ok = false;
    auto mlines = read_lines("input_data/M_" + std::to_string(f) + "_D" + std::to_string(D) + ".txt", ok);
    if (!ok) return false;
    std::vector<double> m;
    for (auto &l : mlines) m.insert(m.end(), l.begin(), l.end());
    if ((long)m.size() < (long)nc * D * D) return false;
    auto slines = read_lines("input_data/shift_data_" + std::to_string(f) + ".txt", ok);
    if (!ok) return false;
    shift.assign((size_t)nc * np2, 0.f);
    if (nc == 1) {
        std::vector<double> all;
        for (auto &l : slines) all.insert(all.end(), l.begin(), l.end());
        if ((int)all.size() < D) return false;
        for (int j = 0; j < D; ++j) shift[j] = (float)all[j];
    } else {
        if ((int)slines.size() < nc) return false;
        for (int c = 0; c < nc; ++c) {
            if ((int)slines[c].size() < D) return false;
            for (int j = 0; j < D; ++j) shift[(size_t)c * np2 + j] = (float)slines[c][j];
        }
    }
    rot.assign((size_t)nc * np2 * D, 0.f);
    for (int c = 0; c < nc; ++c)
        for (int i = 0; i < D; ++i)
            for (int j = 0; j < D; ++j) rot[(size_t)c * np2 * D + (size_t)j * D + i] = (float)m[((size_t)c * D + i) * D + j];
    shuf.assign((size_t)nc * np2, 0);
    if (uses_shuffle(f)) {
        auto sh = read_lines("input_data/shuffle_data_" + std::to_string(f) + "_D" + std::to_string(D) + ".txt", ok);
        if (!ok) return false;
        std::vector<double> all;
        for (auto &l : sh) all.insert(all.end(), l.begin(), l.end());
        if ((long)all.size() < (long)nc * D) return false;
        for (int c = 0; c < nc; ++c)
            for (int j = 0; j < D; ++j) shuf[(size_t)c * np2 + j] = (int)all[(size_t)c * D + j];
    }
    return true;
}

std::string ea_parameters(double CR, double F, int strategy)
{
    static const char *names[9] = {"_current/1/bin", "_current/2/bin", "_current-to-best/1/bin",
                                   "_current-to-best/2/bin", "_rand/1/bin", "_rand/2/bin",
                                   "_best/1/bin", "_best/2/bin", "_current_to_rand/1/bin"};
    std::ostringstream a, b;  // DE_CUDA::GetParameters (CUDA_EA_library/DE_CUDA.cc:18-55)
    a << CR;
    b << F;
    return "CR/F=" + a.str() + "/" + b.str() + (strategy >= 0 && strategy <= 8 ? names[strategy] : "");
}

#define CK(x)                                                                                  \
    do {                                                                                       \
        cudaError_t e_ = (x);                                                                  \
        if (e_ != cudaSuccess) {                                                               \
            std::fprintf(stderr, "speo_gpu: %s: %s\n", #x, cudaGetErrorString(e_));            \
            return 1;                                                                          \
        }                                                                                      \
    } while (0)
#define SK(x)                                                                                  \
    do {                                                                                       \
        int s_ = (x);                                                                          \
        if (s_ != SPEO_OK) {                                                                   \
            std::fprintf(stderr, "speo_gpu: %s: %s\n", #x, speo_last_error());                 \
            return 1;                                                                          \
        }                                                                                      \
    } while (0)

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// One (function, run): IslandEA::Initilize + Execute + RecordDisplayUnit + PrintResult.
int run_one(const Params &p, int fid, int run, const std::string &csv)
{
    const int N = p.GPU_num, P = p.island_size, D = p.dim;
    int np2 = 1;
    while (np2 < D) np2 <<= 1;
    if (np2 < 32) np2 = 32;
    std::vector<float> h_shift, h_rot;
    std::vector<int> h_shuf;
    if (!load_instance(fid, D, np2, h_shift, h_rot, h_shuf)) {
        std::fprintf(stderr, "speo_gpu: cannot read input_data for function %d at D=%d\n", fid, D);
        return 1;
    }
    const size_t rows = (size_t)N * P;
    float *pop = nullptr, *cand = nullptr, *pfit = nullptr, *cfit = nullptr, *shift = nullptr, *rot = nullptr;
    int *shuf = nullptr, *perm = nullptr, *best = nullptr, *nsub_d = nullptr;
    void *rng = nullptr, *info = nullptr, *state = nullptr;
    double *x64 = nullptr, *o64 = nullptr, *m64 = nullptr, *f64 = nullptr;
    const int max_sub = P / 4;
    speo_archipelago arch{};
    arch.n_islands = N;
    arch.island_size = P;
    arch.dim = D;
    arch.ld = np2;
    arch.migration_size = p.migration_size;
    arch.buffer_capacity = p.buffer_capacity;
    arch.buffer_policy = buffer_policy(p.buffer_manage);
    arch.regroup_option = regroup_option(p.regroup_option);
    arch.migration_rate = (float)p.migration_rate;
    arch.seed = (uint64_t)(fid + 1) * 1000003u + (uint64_t)run;
    const size_t state_bytes = speo_archipelago_state_bytes(&arch);
    CK(cudaMalloc(&pop, sizeof(float) * rows * np2));
    CK(cudaMalloc(&cand, sizeof(float) * rows * np2));
    CK(cudaMemset(cand, 0, sizeof(float) * rows * np2));
    CK(cudaMalloc(&pfit, sizeof(float) * rows));
    CK(cudaMalloc(&cfit, sizeof(float) * rows));
    CK(cudaMalloc(&shift, sizeof(float) * h_shift.size()));
    CK(cudaMalloc(&rot, sizeof(float) * h_rot.size()));
    CK(cudaMalloc(&shuf, sizeof(int) * h_shuf.size()));
    CK(cudaMalloc(&perm, sizeof(int) * rows));
    CK(cudaMalloc(&best, sizeof(int) * (size_t)N * max_sub));
    CK(cudaMalloc(&nsub_d, sizeof(int) * N));
    CK(cudaMalloc(&rng, (size_t)N * SPEO_RNG_STATE_BYTES));
    CK(cudaMalloc(&info, sizeof(speo_de_info_f32) * (size_t)N * max_sub));
    CK(cudaMalloc(&state, state_bytes));
    CK(cudaMemcpy(shift, h_shift.data(), sizeof(float) * h_shift.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(rot, h_rot.data(), sizeof(float) * h_rot.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(shuf, h_shuf.data(), sizeof(int) * h_shuf.size(), cudaMemcpyHostToDevice));
    SK(speo_archipelago_init(&arch, state, perm, nsub_d, p.subisland_num, nullptr));

    const bool dynamic_de = p.configure_EA == "dynamic";
    std::vector<int> nsub(N, p.subisland_num), seeds(N);
    std::vector<speo_de_info_f32> h_info((size_t)max_sub);
    auto configure = [&](int i, uint32_t event) -> int {  // DE_CUDA::ConfigureEA (DE_CUDA.cc:89-118)
        SK(speo_configure_de_f32(h_info.data(), nsub[i], P, 0.5f, 0.9f, 4, dynamic_de ? 1 : 0,
                                 ((uint64_t)seeds[i] << 32) | event));
        CK(cudaMemcpy(static_cast<speo_de_info_f32 *>(info) + (size_t)i * max_sub, h_info.data(),
                      sizeof(speo_de_info_f32) * nsub[i], cudaMemcpyHostToDevice));
        return 0;
    };
    auto island = [&](int i) {
        speo_island_info ii;
        ii.island_size = P;
        ii.subisland_num = nsub[i];
        ii.permutated_index = perm + (size_t)i * P;
        return ii;
    };
    auto problem = [&](int i) {
        speo_problem_info_f32 pi{};
        pi.dim = D;
        pi.function_ID = fid;
        pi.run_ID = run;
        pi.max_base_FEs = p.max_base_FEs;
        pi.seed = seeds[i];
        pi.computing_time = p.computing_time;
        pi.max_bound = (float)p.max_bound;
        pi.min_bound = (float)p.min_bound;
        return pi;
    };
    auto popn = [&](float *x, float *f, int i) {
        speo_population_f32 q;
        q.elements = x + (size_t)i * P * np2;
        q.fitness_value = f + (size_t)i * P;
        return q;
    };
    char *rng_b = static_cast<char *>(rng);
    for (int i = 0; i < N; ++i) {  // IslandEA::Initilize (island_EA.cc:33-43), node_ID = island i
        seeds[i] = (i + fid) * (run + fid);
        SK(API_Initilize_f32(popn(pop, pfit, i), reinterpret_cast<speo_rng_state *>(rng_b + (size_t)i * SPEO_RNG_STATE_BYTES),
                             island(i), problem(i)));
        API_evaluateFitness_f32(pfit + (size_t)i * P, nullptr, nullptr, pop + (size_t)i * P * np2, shift, rot, shuf,
                                nullptr, nullptr, nullptr, P, D, 0.f, fid);
        if (configure(i, 0)) return 1;
    }
    SK(API_CheckCUDAError());

    // IslandEA::Execute (island_EA.cc:78-113)
    const long long total_FEs = (long long)p.max_base_FEs * D / N;
    long long current_FEs = P;
    uint32_t generation = 0;
    double comm = 0;
    const double t0 = now_s();
    const bool dyn_regroup = arch.regroup_option == SPEO_REGROUP_DYNAMIC_ORDERED ||
                             arch.regroup_option == SPEO_REGROUP_DYNAMIC_RANDOM;
    while (current_FEs < total_FEs) {
        for (int i = 0; i < N; ++i) {  // RunEA -> DE_CUDA::Run (DE_CUDA.cc:200-216)
            speo_rng_state *r = reinterpret_cast<speo_rng_state *>(rng_b + (size_t)i * SPEO_RNG_STATE_BYTES);
            SK(API_DE_GenerateNewPopulation_f32(popn(cand, cfit, i), popn(pop, pfit, i), best + (size_t)i * max_sub,
                                                island(i), static_cast<speo_de_info_f32 *>(info) + (size_t)i * max_sub,
                                                r, problem(i)));
            API_evaluateFitness_f32(cfit + (size_t)i * P, nullptr, nullptr, cand + (size_t)i * P * np2, shift, rot,
                                    shuf, nullptr, nullptr, nullptr, P, D, 0.f, fid);
            SK(API_DE_SelectSurvival_f32(popn(pop, pfit, i), popn(cand, cfit, i), island(i), problem(i)));
        }
        CK(cudaDeviceSynchronize());
        const double tm = now_s();
        if (generation % (uint32_t)p.interval == 0) {
            SK(speo_migrate_out(&arch, state, pop, pfit, perm, nsub_d, generation, nullptr));
            if (dyn_regroup) {  // RegroupIslands -> ConfigureEA (migrate.cc:160-161, 174-175)
                CK(cudaMemcpy(nsub.data(), nsub_d, sizeof(int) * N, cudaMemcpyDeviceToHost));
                for (int i = 0; i < N; ++i)
                    if (configure(i, generation + 1)) return 1;
            }
        }
        SK(speo_migrate_in(&arch, state, pop, pfit, generation, nullptr));
        CK(cudaDeviceSynchronize());
        comm += now_s() - tm;
        ++generation;
        current_FEs += P;
    }
    SK(API_CheckCUDAError());
    const double elapsed = now_s() - t0;

    // RecordDisplayUnit + MergeResults: the best row over the islands, re-evaluated in FP64
    std::vector<float> h_fit(rows);
    CK(cudaMemcpy(h_fit.data(), pfit, sizeof(float) * rows, cudaMemcpyDeviceToHost));
    size_t bi = 0;
    for (size_t r = 1; r < rows; ++r)
        if (h_fit[r] < h_fit[bi]) bi = r;
    std::vector<float> xrow(np2);
    CK(cudaMemcpy(xrow.data(), pop + bi * np2, sizeof(float) * np2, cudaMemcpyDeviceToHost));
    std::vector<double> x(np2), o(h_shift.begin(), h_shift.end()), m(h_rot.begin(), h_rot.end());
    for (int j = 0; j < np2; ++j) x[j] = xrow[j];
    CK(cudaMalloc(&x64, sizeof(double) * np2));
    CK(cudaMalloc(&o64, sizeof(double) * o.size()));
    CK(cudaMalloc(&m64, sizeof(double) * m.size()));
    CK(cudaMalloc(&f64, sizeof(double)));
    CK(cudaMemcpy(x64, x.data(), sizeof(double) * np2, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(o64, o.data(), sizeof(double) * o.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(m64, m.data(), sizeof(double) * m.size(), cudaMemcpyHostToDevice));
    API_evaluateFitness(f64, nullptr, nullptr, x64, o64, m64, shuf, nullptr, nullptr, nullptr, 1, D, 0.0, fid);
    SK(API_CheckCUDAError());
    double best_fitness = 0;
    CK(cudaMemcpy(&best_fitness, f64, sizeof(double), cudaMemcpyDeviceToHost));
    std::printf("Run: %d, Time: %.3lf s, Best fitness: %.9lf\n", run, elapsed, best_fitness);

    // IslandEA::PrintResult (island_EA.cc:146-171)
    std::ofstream file(csv, std::ios::app);
    const long long total_FEs_all = (long long)p.max_base_FEs * D;
    const int subisland_size = dyn_regroup ? -1 : P / p.subisland_num;
    file << fid << ',' << run << ',' << D << ',' << best_fitness << ',' << elapsed << ',' << comm / elapsed << ','
         << total_FEs_all << ',' << p.node_num << ',' << p.GPU_num << ',' << N << ',' << (long long)N * P << ','
         << subisland_size << ',' << p.interval << ',' << p.migration_size << ',' << p.migration_rate << ','
         << p.buffer_capacity << ',' << p.migration_topology << ',' << p.buffer_manage << ',' << p.regroup_option
         << ',' << p.configure_EA << ',' << ea_parameters(0.9, 0.5, 4) << std::endl;

    for (void *q : {(void *)pop, (void *)cand, (void *)pfit, (void *)cfit, (void *)shift, (void *)rot, (void *)shuf,
                    (void *)perm, (void *)best, (void *)nsub_d, rng, info, state, (void *)x64, (void *)o64,
                    (void *)m64, (void *)f64})
        cudaFree(q);
    return 0;
}

}  // namespace

int main(int argc, char **argv)
{
    Params p;
    if (int e = set_parameters(p, argc, argv)) return e;
    const double start = now_s();
    // IslandEA::CheckAndCreatRecordFile (island_EA.cc:13-31)
    const std::string csv = "./Results/SPEO_GPU.csv";
    mkdir("./Results", 0755);
    {
        std::ifstream exist(csv);
        if (!exist) {
            std::ofstream f(csv);
            f << "function_ID,run_ID,dim,best_fitness,time_period,communication_percentage,total_FEs,node_num,"
                 "GPU_num,island_num,total_pop_size,subisland_size,interval,migration_size,migration_rate,"
                 "buffer_capacity,migration_topology,buffer_manage,regroup_option,configure_EA,EA_parameters"
              << std::endl;
        }
    }
    for (int fid : p.functions)  // ConstructAndExecuteIslandModule (main.cc:124-150); this process is node 0
        for (int run : p.runs)
            if (int e = run_one(p, fid, run, csv)) return e;
    std::printf("Total Elapsed time: %f seconds\n", now_s() - start);
    return 0;
}
