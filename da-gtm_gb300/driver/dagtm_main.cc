// dagtm_main.cc -- the `dagtm` command with the reference's options, screen
// output and HDF5 files, running the EM step on one GB300 through the C ABI.
//
// It follows the control flow of dagtm/dagtm.cxx (main, :714-2633) for one
// process: options (:719-891), reading T/id/lb (:1070-1101), random set-up or
// restart (:1104-1213), the temperature loop with the EXP, LINEAR and AUTO
// schedules and the hierarchical expansion of EXP (-H, :1508-2206),
// checkpoints (:1609-1687), interpolation (:1247-1295) and the output file
// (:2342-2552).  The MPI grid (-z) has nothing to do on one GPU.  Extra
// options: -F form (fp64 | fp32 | bf16x3, default fp64),
// -G width (basis-function width factor, default 2 as the reference
// hard-codes at :1119), -Q solver (cholesky | svd, default svd as the
// reference's dagtm_solve2).
#include "../../include/dagtm_gb300.h"
#include "h5lite.h"

#include <cfloat>
#include <cstdarg>
#include <cctype>
#include <map>
#include <algorithm>
#include <cmath>
#include <csignal>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <getopt.h>
#include <string>
#include <sys/times.h>
#include <unistd.h>
#include <vector>

namespace {

volatile sig_atomic_t g_force_checkpoint = 0;
void on_signal(int) { g_force_checkpoint = 1; }  // dagtm/dagtm.cxx:2628-2633

FILE *g_log = stdout;

[[noreturn]] void die(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    fprintf(stderr, "dagtm: ");
    vfprintf(stderr, fmt, ap);
    fprintf(stderr, "\n");
    va_end(ap);
    exit(EXIT_FAILURE);
}

void check(int rc, const char *what)
{
    if (rc != DGTM_OK)
        die("%s failed: %s", what, dgtm_last_error_string());
}

// ---------------------------------------------------------------- host math
// MT19937 (Matsumoto & Nishimura), seeded as gsl_rng_set does (0 -> 4357).
struct MT {
    uint32_t mt[624];
    int i = 624;
    explicit MT(unsigned long seed)
    {
        if (seed == 0)
            seed = 4357;
        mt[0] = (uint32_t) seed;
        for (int k = 1; k < 624; k++)
            mt[k] = (uint32_t) (1812433253UL * (mt[k - 1] ^ (mt[k - 1] >> 30)) + (uint32_t) k);
    }
    uint32_t next()
    {
        if (i >= 624) {
            for (int k = 0; k < 624; k++) {
                const uint32_t y = (mt[k] & 0x80000000u) | (mt[(k + 1) % 624] & 0x7fffffffu);
                mt[k] = mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
            }
            i = 0;
        }
        uint32_t y = mt[i++];
        y ^= y >> 11;
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        y ^= y >> 18;
        return y;
    }
    double uniform() { return next() / 4294967296.0; }
};

// Cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (row-major):
// on return a holds the eigenvalues on its diagonal and V the eigenvectors.
void jacobi_eig(int n, std::vector<double> &a, std::vector<double> &V)
{
    V.assign((size_t) n * n, 0.0);
    for (int i = 0; i < n; i++)
        V[(size_t) i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                const double v = a[(size_t) i * n + j] * a[(size_t) i * n + j];
                tot += v;
                if (i != j)
                    off += v;
            }
        if (off <= 1e-32 * tot)
            break;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                const double apq = a[(size_t) p * n + q];
                if (apq == 0.0)
                    continue;
                const double th = (a[(size_t) q * n + q] - a[(size_t) p * n + p]) / (2.0 * apq);
                const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {
                    const double akp = a[(size_t) k * n + p], akq = a[(size_t) k * n + q];
                    a[(size_t) k * n + p] = c * akp - s * akq;
                    a[(size_t) k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    const double apk = a[(size_t) p * n + k], aqk = a[(size_t) q * n + k];
                    a[(size_t) p * n + k] = c * apk - s * aqk;
                    a[(size_t) q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; k++) {
                    const double vp = V[(size_t) k * n + p], vq = V[(size_t) k * n + q];
                    V[(size_t) k * n + p] = c * vp - s * vq;
                    V[(size_t) k * n + q] = s * vp + c * vq;
                }
            }
    }
}

// Least squares (A^T A) X = A^T B through the eigen-decomposition of A^T A,
// exactly-zero eigenvalues dropped (comm/comm.c:1247-1294, dagtm_solve).
void solve_ls(int m, int n, int k, const std::vector<double> &A, const std::vector<double> &B,
              std::vector<double> &X)
{
    std::vector<double> U((size_t) n * n, 0.0), AB((size_t) n * k, 0.0), V;
    for (int r = 0; r < m; r++)
        for (int i = 0; i < n; i++) {
            const double a = A[(size_t) r * n + i];
            for (int j = 0; j < n; j++)
                U[(size_t) i * n + j] += a * A[(size_t) r * n + j];
            for (int j = 0; j < k; j++)
                AB[(size_t) i * k + j] += a * B[(size_t) r * k + j];
        }
    jacobi_eig(n, U, V);
    X.assign((size_t) n * k, 0.0);
    std::vector<double> w(n);
    for (int c = 0; c < k; c++) {
        for (int i = 0; i < n; i++) {
            double acc = 0.0;
            for (int r = 0; r < n; r++)
                acc += V[(size_t) r * n + i] * AB[(size_t) r * k + c];
            double lam = U[(size_t) i * n + i];
            w[i] = (lam != 0.0) ? acc / lam : 0.0;
        }
        for (int r = 0; r < n; r++) {
            double acc = 0.0;
            for (int i = 0; i < n; i++)
                acc += V[(size_t) r * n + i] * w[i];
            X[(size_t) r * k + c] = acc;
        }
    }
}

double sqdist(const double *a, const double *b, int d)
{
    double s = 0.0;
    for (int i = 0; i < d; i++) {
        const double t = a[i] - b[i];
        s += t * t;
    }
    return s;
}

// Regular grid in [-1, 1]^L, x fastest (comm/comm.c:1453-1504).
std::vector<double> latent_grid(int L, int g)
{
    const int total = (int) lround(pow(g, L));
    std::vector<double> X((size_t) total * L);
    for (int idx = 0; idx < total; idx++) {
        int r = idx;
        for (int l = 0; l < L; l++) {
            X[(size_t) idx * L + l] = (r % g) * (2 / (double) (g - 1)) + -1.0;
            r /= g;
        }
    }
    return X;
}

// X and FI for K = gx^L latent points and M = gf^L centres of width s x spacing
// (comm/comm.c:992-1103, dagtm_stp; dagtm_gbf :1506-1536).
void setup_grid(int L, int K, int M, double s, std::vector<double> &X, std::vector<double> &FI)
{
    const int gx = (int) lround(pow(K, 1.0 / L)), gf = (int) lround(pow(M, 1.0 / L));
    if (lround(pow(gx, L)) != K)
        die("K = %d is not acceptable (not a perfect %d-th power)", K, L);
    if (lround(pow(gf, L)) != M || gf < 2)
        die("M = %d is not acceptable (not a perfect %d-th power of at least 2)", M, L);
    X = latent_grid(L, gx);
    std::vector<double> MU = latent_grid(L, gf);
    for (double &v : MU)
        v *= (double) gf / (gf - 1);
    const double sigma = s * (MU[1 * L] - MU[0]);
    FI.assign((size_t) K * (M + 1), 1.0);
    for (int k = 0; k < K; k++)
        for (int j = 0; j < M; j++)
            FI[(size_t) k * (M + 1) + j] =
                exp(sqdist(&X[(size_t) k * L], &MU[(size_t) j * L], L) * (-0.5 / (sigma * sigma)));
}

struct Opts {
    int K = 125, L = 3, M = 8, maxloop = 0, period = 100, verbose = 0, Kmax = 32768;
    double alpha = 0.99, delta = 0.1, eps = 1e-6, eps2 = 1e-3, start_temp = 1.0, width = 2.0;
    bool need_ctemp = true, isDA = true, checkpointing = true, log_progress = false,
         save_R = false, log_file = false, interpolation = false, hda = false;
    int schedule = 0;  // 0 EXP, 1 LINEAR, 2 AUTO
    unsigned long seed = 0;
    std::string in = "INPUT.h5", out, restart, prefix = "ckp.";
    std::string dT = "T", dX = "X", dFI = "FI", dW = "W", dY = "Y", dR = "R", dbeta = "beta",
                dM = "M", did = "id", dlb = "lb", dtemp = "temp", diter = "iter", dseed = "seed",
                dqual = "qual";
    int form = DGTM_FP64, solver = DGTM_SOLVE_SVD;
    bool rd_output = false;  // -J
};

void help()
{
    static const char *lines[] = {
        "-a number    : alpha (default: 0.99)",
        "-b name      : dataset name for beta (default: beta)",
        "-B name      : dataset name for label (default: lb)",
        "-c schedule  : cooling schedule [auto|exp|linear] (default : exp)",
        "-e number    : precision (default: 1e-6)",
        "-E number    : log-likelihood gain that confirms an HDA expansion (default: 1e-3)",
        "-f dataset   : dataset name for FI (default: FI)",
        "-F form      : arithmetic [fp64|fp32|bf16x3] (default: fp64)",
        "-G number    : basis-function width factor (default: 2)",
        "-h           : show help",
        "-H           : hierarchical DA (EXP schedule: grow K at critical temperatures)",
        "-i filename  : input HDF5 filename",
        "-I           : interpolation",
        "-j number    : maximum number of iterations",
        "-J           : after a -j stop, write M and R from R o D, as the reference does",
        "-k number    : largest K of the hierarchical DA (default: 32768)",
        "-K number    : number of latent data K (eg, 100, 1k, 1M)",
        "-l           : log to file",
        "-L number    : latent dimension",
        "-m           : EM",
        "-M number    : number of model",
        "-n           : disable checkpointing",
        "-o filename  : output HDF5 filename",
        "-p           : log progress",
        "-P number    : checkpointing per num. loop",
        "-Q solver    : M-step solver [svd|cholesky] (default: svd)",
        "-r filename  : restarting",
        "-R           : save responsibilities",
        "-s number    : seed",
        "-S number    : start temp",
        "-t dataset   : dataset name for T (default: T)",
        "-v number    : set verbose level",
        "-w prefix    : checkpointing file prefix",
        "-W dataset   : dataset name for W (default: W)",
        "-x dataset   : dataset name for X (default: X)",
        "-z PxQ       : compute grid (ignored: one GPU)",
        nullptr};
    fprintf(stderr, "usage: dagtm [OPTIONS]\n");
    for (const char **p = lines; *p; p++)
        fprintf(stderr, "\t%s\n", *p);
}

Opts parse(int argc, char **argv)
{
    Opts o;
    int c;
    opterr = 0;
    while ((c = getopt(argc, argv, "a:b:B:c:e:E:f:F:g:G:hHi:Ij:Jk:K:lL:mM:no:pP:Q:r:Rs:S:t:v:w:W:x:z:")) != -1) {
        switch (c) {
        case 'a': o.alpha = atof(optarg); break;
        case 'b': o.dbeta = optarg; break;
        case 'B': o.dlb = optarg; break;
        case 'c':
            if (!strcasecmp(optarg, "exp"))
                o.schedule = 0;
            else if (!strcasecmp(optarg, "linear"))
                o.schedule = 1;
            else if (!strcasecmp(optarg, "auto"))
                o.schedule = 2;
            else
                die("unknown cooling schedule: %s", optarg);
            break;
        case 'e': o.eps = atof(optarg); break;
        case 'E': o.eps2 = atof(optarg); break;
        case 'f': o.dFI = optarg; break;
        case 'F':
            if (!strcmp(optarg, "fp64"))
                o.form = DGTM_FP64;
            else if (!strcmp(optarg, "fp32"))
                o.form = DGTM_FP32;
            else if (!strcmp(optarg, "bf16x3"))
                o.form = DGTM_BF16X3;
            else
                die("unknown form: %s", optarg);
            break;
        case 'g':
            if (strcasecmp(optarg, "sweep") != 0)
                die("grid type %s is not part of this build (sweep only)", optarg);
            break;
        case 'G': o.width = atof(optarg); break;
        case 'h': help(); exit(EXIT_SUCCESS);
        case 'H': o.hda = !o.hda; break;
        case 'i': o.in = optarg; break;
        case 'I': o.interpolation = true; break;
        case 'j': o.maxloop = atoi(optarg); break;
        case 'J': o.rd_output = !o.rd_output; break;
        case 'k': o.Kmax = atoi(optarg); break;
        case 'K': {
            float num = 0, unit = 1;
            char ch = 0;
            if (sscanf(optarg, "%f%c", &num, &ch) >= 1) {
                if (ch == 'k' || ch == 'K')
                    unit = 1000;
                else if (ch == 'm' || ch == 'M')
                    unit = 1000 * 1000;
                else if (ch == 'g' || ch == 'G')
                    unit = 1000 * 1000 * 1000;
            }
            o.K = (int) (num * unit);
        } break;
        case 'l': o.log_file = !o.log_file; break;
        case 'L': o.L = atoi(optarg); break;
        case 'm': o.isDA = !o.isDA; break;
        case 'M': o.M = atoi(optarg); break;
        case 'n': o.checkpointing = false; break;
        case 'o': o.out = optarg; break;
        case 'p': o.log_progress = !o.log_progress; break;
        case 'P': o.period = atoi(optarg); break;
        case 'Q':
            if (!strcmp(optarg, "svd"))
                o.solver = DGTM_SOLVE_SVD;
            else if (!strcmp(optarg, "cholesky"))
                o.solver = DGTM_SOLVE_CHOLESKY;
            else
                die("unknown solver: %s", optarg);
            break;
        case 'r': o.restart = optarg; break;
        case 'R': o.save_R = !o.save_R; break;
        case 's': o.seed = (unsigned long) atoi(optarg); break;
        case 'S':
            o.start_temp = atof(optarg);
            o.need_ctemp = false;
            break;
        case 't': o.dT = optarg; break;
        case 'v': o.verbose = atoi(optarg); break;
        case 'w': o.prefix = optarg; break;
        case 'W': o.dW = optarg; break;
        case 'x': o.dX = optarg; break;
        case 'z': break;  // the P x Q grid has nothing to do on one GPU
        case '?':
            if (isprint(optopt))
                fprintf(stderr, "Unknown option `-%c'.\n", optopt);
            else
                fprintf(stderr, "Unknown option character `\\x%x'.\n", optopt);
            exit(1);
        default: abort();
        }
    }
    return o;
}

const h5lite::Dataset &need(const std::map<std::string, h5lite::Dataset> &f, const std::string &name,
                            const std::string &file)
{
    auto it = f.find(name);
    if (it == f.end())
        die("dataset %s not found in %s", name.c_str(), file.c_str());
    return it->second;
}

double scalar(const std::map<std::string, h5lite::Dataset> &f, const std::string &name,
              const std::string &file)
{
    const h5lite::Dataset &d = need(f, name, file);
    if (d.is_int)
        return d.i64.empty() ? 0.0 : (double) d.i64[0];
    return d.f64.empty() ? 0.0 : d.f64[0];
}

}  // namespace

// `dagtm --h5dump file.h5`: list the datasets (name, class, shape, sum) the
// driver can read, without touching the GPU.
int h5dump(const char *path)
{
    std::map<std::string, h5lite::Dataset> f;
    std::string err;
    if (!h5lite::read_file(path, f, err)) {
        fprintf(stderr, "dagtm: %s\n", err.c_str());
        return 1;
    }
    for (auto &kv : f) {
        const h5lite::Dataset &d = kv.second;
        double sum = 0.0;
        if (d.is_int)
            for (int64_t v : d.i64)
                sum += (double) v;
        else
            for (double v : d.f64)
                sum += v;
        printf("%s %s", kv.first.c_str(), d.is_int ? "int" : "float");
        for (uint64_t n : d.dims)
            printf(" %llu", (unsigned long long) n);
        printf(" sum=%.17g\n", sum);
    }
    return 0;
}

int main(int argc, char **argv)
{
    if (argc == 3 && !strcmp(argv[1], "--h5dump"))
        return h5dump(argv[2]);
    Opts o = parse(argc, argv);
    if (o.log_file) {
        g_log = fopen("dagtm.P000.log", "w");  // comm/comm.h:89 names one log per rank
        if (!g_log)
            die("cannot open dagtm.P000.log");
    }
    struct tms st_cpu, en_cpu;
    const clock_t st_time = times(&st_cpu);
    const long clk_tck = sysconf(_SC_CLK_TCK);

    // ---- input (dagtm/dagtm.cxx:919-930,1070-1101)
    std::map<std::string, h5lite::Dataset> inp;
    std::string err;
    if (!h5lite::read_file(o.in, inp, err))
        die("%s", err.c_str());
    const h5lite::Dataset &Td = need(inp, o.dT, o.in);
    if (Td.dims.size() != 2 || Td.is_int)
        die("dataset %s must be a 2-D floating-point matrix", o.dT.c_str());
    const int N = (int) Td.dims[0], D = (int) Td.dims[1];
    const std::vector<double> &T = Td.f64;
    std::vector<int32_t> id, lb;
    if (inp.count(o.did) && inp[o.did].is_int)
        for (int64_t v : inp[o.did].i64)
            id.push_back((int32_t) v);
    if (inp.count(o.dlb) && inp[o.dlb].is_int)
        for (int64_t v : inp[o.dlb].i64)
            lb.push_back((int32_t) v);

    signal(SIGCHLD, on_signal);  // dagtm/dagtm.cxx:978

    // ---- set-up or restart (dagtm/dagtm.cxx:1104-1213)
    int K = o.K, L = o.L, M = o.M, nloop = 0, maxloop = o.maxloop;
    std::vector<double> X, FI, W, Y;
    double beta = 0.1, temp = 1.0, start_temp = o.start_temp, first_ctemp = 1.0;
    unsigned long seed = o.seed;
    if (o.restart.empty()) {
        setup_grid(L, K, M, o.width, X, FI);
        // dagtm_mpi_mean / dagtm_mpi_sd (comm/mpicomm.c:686-730)
        std::vector<double> mu(D, 0.0), sd(D, 0.0);
        for (int n = 0; n < N; n++)
            for (int d = 0; d < D; d++)
                mu[d] += T[(size_t) n * D + d];
        for (int d = 0; d < D; d++)
            mu[d] *= 1.0 / N;
        for (int n = 0; n < N; n++)
            for (int d = 0; d < D; d++) {
                const double c = T[(size_t) n * D + d] - mu[d];
                sd[d] += c * c;
            }
        for (int d = 0; d < D; d++)
            sd[d] = sqrt(sd[d] * (1.0 / (N - 1)));
        // dagtm_yrnd2 + dagtm_solve + dagtm_bi (comm/comm.c:1118-1185,1401-1448)
        if (seed == 0)
            seed = (unsigned long) time(nullptr);
        MT rng(seed);
        std::vector<double> Yr((size_t) K * D);
        for (int k = 0; k < K; k++)
            for (int d = 0; d < D; d++) {
                const double dev = sd[d] * 6;
                const double rnd = ceil(rng.uniform() / 1e-15) * 1e-15;
                Yr[(size_t) k * D + d] = 2 * dev * rnd - dev + mu[d];
            }
        solve_ls(K, M + 1, D, FI, Yr, W);
        if (K > 1000) {
            beta = 0.1;
        } else {
            long double mean = 0;
            for (int j = 0; j < K; j++) {
                double mn = DBL_MAX;
                for (int i = 0; i < K; i++)
                    if (i != j)
                        mn = fmin(mn, sqdist(&Yr[(size_t) i * D], &Yr[(size_t) j * D], D));
                mean += (mn - mean) / (j + 1);
            }
            const double m = (double) mean;
            beta = 2 / (m == 0 ? 1 : m);
        }
        Y.assign((size_t) K * D, 0.0);
        for (int k = 0; k < K; k++)
            for (int m = 0; m < M + 1; m++)
                for (int d = 0; d < D; d++)
                    Y[(size_t) k * D + d] += FI[(size_t) k * (M + 1) + m] * W[(size_t) m * D + d];
        if (o.isDA) {
            if (o.need_ctemp) {
                // dagtm_mpi_ctemp (comm/mpicomm.c:511-559)
                std::vector<double> S((size_t) D * D, 0.0), V, row(D);
                double csum = 0.0;
                for (int n = 0; n < N; n++) {
                    for (int d = 0; d < D; d++) {
                        row[d] = T[(size_t) n * D + d] - mu[d];
                        csum += row[d] * row[d];
                    }
                    for (int i = 0; i < D; i++)
                        for (int j = 0; j < D; j++)
                            S[(size_t) i * D + j] += row[i] * row[j];
                }
                jacobi_eig(D, S, V);
                double lmax = S[0];
                for (int d = 1; d < D; d++)
                    lmax = fmax(lmax, S[(size_t) d * D + d]);
                first_ctemp = lmax / N * ((double) N * D / csum);
                start_temp = first_ctemp / pow(o.alpha, 10);
            }
            temp = start_temp;
        }
    } else {
        std::map<std::string, h5lite::Dataset> ck;
        if (!h5lite::read_file(o.restart, ck, err))
            die("%s", err.c_str());
        X = need(ck, o.dX, o.restart).f64;
        FI = need(ck, o.dFI, o.restart).f64;
        Y = need(ck, o.dY, o.restart).f64;
        const auto &xd = need(ck, o.dX, o.restart).dims;
        const auto &fd = need(ck, o.dFI, o.restart).dims;
        K = (int) xd[0];
        L = (int) xd[1];
        M = (int) fd[1] - 1;
        beta = scalar(ck, o.dbeta, o.restart);
        temp = scalar(ck, o.dtemp, o.restart);
        nloop = (int) scalar(ck, o.diter, o.restart);
        seed = (unsigned long) scalar(ck, o.dseed, o.restart);
        start_temp = temp;
        if (maxloop)
            maxloop = nloop + maxloop;  // dagtm/dagtm.cxx:1208-1211
    }

    dgtm_ctx *ctx = nullptr;
    check(dgtm_ctx_create(N, D, K, M + 1, T.data(), D, FI.data(), M + 1, o.form, &ctx),
          "dgtm_ctx_create");
    check(dgtm_set_solver(ctx, o.solver), "dgtm_set_solver");
    check(dgtm_set_Y(ctx, Y.data(), D), "dgtm_set_Y");

    auto write_output = [&](const std::vector<double> &Mout, double qual, bool include_R,
                            bool rd = false) {
        h5lite::Writer w;
        std::map<std::string, h5lite::Dataset> old;
        w.add_f64(o.dT, {(uint64_t) N, (uint64_t) D}, T.data());
        w.add_f64(o.dM, {(uint64_t) N, (uint64_t) L}, Mout.data());
        w.add_f64(o.dX, {(uint64_t) K, (uint64_t) L}, X.data());
        w.add_f64(o.dFI, {(uint64_t) K, (uint64_t) M + 1}, FI.data());
        w.add_f64(o.dY, {(uint64_t) K, (uint64_t) D}, Y.data());
        if (!W.empty())
            w.add_f64(o.dW, {(uint64_t) M + 1, (uint64_t) D}, W.data());
        if (include_R) {
            std::vector<double> R((size_t) K * N);
            if (rd)
                check(dgtm_get_RD_block(ctx, 0, K, 0, N, R.data(), N), "dgtm_get_RD_block");
            else
                check(dgtm_get_R_block(ctx, 0, K, 0, N, R.data(), N), "dgtm_get_R_block");
            w.add_f64(o.dR, {(uint64_t) K, (uint64_t) N}, R.data());
        }
        w.add_scalar_f64(o.dbeta, beta);
        w.add_scalar_f64(o.dtemp, temp);
        w.add_scalar_i32(o.diter, nloop);
        w.add_scalar_i32(o.dseed, (int32_t) seed);
        w.add_scalar_f64(o.dqual, qual);
        if (!id.empty())
            w.add_i32(o.did, {(uint64_t) id.size()}, id.data());
        if (!lb.empty())
            w.add_i32(o.dlb, {(uint64_t) lb.size()}, lb.data());
        return w;
    };

    // ---- interpolation (dagtm/dagtm.cxx:1247-1295)
    if (o.interpolation) {
        if (o.restart.empty())
            fprintf(stderr, "dagtm: interpolating without a checkpoint file\n");
        if (o.out.empty())
            die("interpolation needs an output file (-o)");
        double llh, nfree;
        check(dgtm_estep(ctx, beta, o.isDA, temp, &llh, &nfree), "dgtm_estep");
        std::vector<double> Mout((size_t) N * L);
        check(dgtm_map(ctx, X.data(), L, Mout.data(), L), "dgtm_map");
        // h5append: keep what the file holds and add M
        std::map<std::string, h5lite::Dataset> old;
        h5lite::Writer w;
        if (access(o.out.c_str(), F_OK) == 0 && h5lite::read_file(o.out, old, err)) {
            for (auto &kv : old) {
                if (kv.first == o.dM)
                    continue;
                if (kv.second.is_int) {
                    std::vector<int32_t> v(kv.second.i64.begin(), kv.second.i64.end());
                    w.add_i32(kv.first, kv.second.dims, v.data());
                } else {
                    w.add_f64(kv.first, kv.second.dims, kv.second.f64.data());
                }
            }
        }
        w.add_f64(o.dM, {(uint64_t) N, (uint64_t) L}, Mout.data());
        if (!w.write(o.out, err))
            die("%s", err.c_str());
        dgtm_ctx_destroy(ctx);
        return 0;
    }

    // ---- the temperature loop (dagtm/dagtm.cxx:1508-2206)
    const int QUEUE = 50;  // INIT_QUEUE_SIZE
    std::vector<double> queue(QUEUE, DBL_MAX), tr_temp, tr_llh, tr_free;
    double llh = 0, nfree = 0, qual = 0, qual_old = 0, diff = DBL_MAX;
    bool isLast = false, stats_current = false;
    std::vector<double> G_last;  // G of the last M-step (AUTO schedule, HDA)
    int lloop = 0;
    // HDA (dagtm/dagtm.cxx:1504-1506, 1937-2124): the expansion state, the
    // per-centre critical temperatures of the last next_ctemp call, and the
    // snapshots written into the output file when progress is logged
    bool ready = false;
    int nexpanded = 0;
    std::vector<double> ctemp_k;
    struct Snap {
        std::string name;
        std::vector<uint64_t> dims;
        std::vector<double> v;
    };
    std::vector<Snap> snaps;

    W.assign((size_t) (M + 1) * D, 0.0);
    bool have_W = false;
    auto hda_step = [&](double qual_before_temp) {
        const double qual_diff = llh - qual_before_temp;
        bool expand = false;
        if (ready) {
            if (qual_diff < o.eps2) {
                fprintf(g_log, "HDA: nothing happened at this temperature, not expanding\n");
                ready = false;
            } else {
                expand = true;
            }
        }
        if (!ready) {
            double ct = 0.0;
            ctemp_k.assign((size_t) K, 0.0);
            check(dgtm_next_ctemp_k(ctx, temp, beta, o.eps,
                                    G_last.empty() ? nullptr : G_last.data(), ctemp_k.data(),
                                    &ct),
                  "dgtm_next_ctemp_k");
            fprintf(g_log, "HDA: ctemp_max : %f\n", ct);
            if (ct >= temp * o.alpha) {
                fprintf(g_log, "HDA: ready to expand\n");
                ready = true;
            }
        }
        if (!expand)
            return;
        ready = false;
        nexpanded++;
        if (!have_W) {
            check(dgtm_get_W(ctx, W.data(), D), "dgtm_get_W");
            have_W = true;
        }
        if (!o.out.empty() && o.log_progress) {
            // dagtm/dagtm.cxx:1980-2096: MAP and the model at this temperature,
            // indexed by the temperature collection's last entry
            const long idx = (long) tr_temp.size() - 1;
            auto name = [&](const std::string &base) { return base + "." + std::to_string(idx); };
            std::vector<double> Mout((size_t) N * L);
            check(dgtm_map(ctx, X.data(), L, Mout.data(), L), "dgtm_map");
            check(dgtm_get_Y(ctx, Y.data(), D), "dgtm_get_Y");
            snaps.push_back({name(o.dM), {(uint64_t) N, (uint64_t) L}, Mout});
            snaps.push_back({name(o.dX), {(uint64_t) K, (uint64_t) L}, X});
            snaps.push_back({name(o.dY), {(uint64_t) K, (uint64_t) D}, Y});
            snaps.push_back({name(o.dFI), {(uint64_t) K, (uint64_t) M + 1}, FI});
            snaps.push_back({name(o.dW), {(uint64_t) M + 1, (uint64_t) D}, W});
            snaps.push_back({name("ctemp"), {(uint64_t) K}, ctemp_k});
            snaps.push_back({name(o.dbeta), {1}, {beta}});
        }
        // dagtm/dagtm.cxx:2110-2144: the latent grid doubles per dimension, X
        // and FI are rebuilt with width factor 2 and the same M, Y = FI W
        const int g = (int) lround(pow((double) K, 1.0 / L)) * 2;
        K = (int) lround(pow((double) g, (double) L));
        fprintf(g_log, "HDA: new K : %d\n", K);
        setup_grid(L, K, M, 2.0, X, FI);
        Y.assign((size_t) K * D, 0.0);
        for (int k = 0; k < K; k++)
            for (int j = 0; j <= M; j++) {
                const double f = FI[(size_t) k * (M + 1) + j];
                for (int d = 0; d < D; d++)
                    Y[(size_t) k * D + d] += f * W[(size_t) j * D + d];
            }
        dgtm_ctx_destroy(ctx);
        ctx = nullptr;
        check(dgtm_ctx_create(N, D, K, M + 1, T.data(), D, FI.data(), M + 1, o.form, &ctx),
              "dgtm_ctx_create");
        check(dgtm_set_solver(ctx, o.solver), "dgtm_set_solver");
        check(dgtm_set_Y(ctx, Y.data(), D), "dgtm_set_Y");
        G_last.clear();
        stats_current = false;
    };
    do {
        if (temp < 1.0) {
            temp = 1.0;
            isLast = true;
        }
        fprintf(g_log, "\nT= %.10g\n", temp);
        const double qual_before_temp = llh;
        std::fill(queue.begin(), queue.end(), DBL_MAX);
        int qnext = 0;
        fprintf(g_log, ">>> %15s %15s %15s %15s %15s %15s\n", "GSEQ", "SEQ", "K", "TEMP", "NFREE", "LLH");
        lloop = 0;
        while (true) {
            check(dgtm_estep(ctx, beta, o.isDA, temp, &llh, &nfree), "dgtm_estep");
            stats_current = true;
            qual_old = qual;
            lloop++;
            nloop++;
            qual = o.isDA ? nfree : llh;
            diff = qual - qual_old;
            fprintf(g_log, "::: %15d %15d %15d %15.7f %15.7f %15.7f %15.7f\n", nloop, lloop, K, temp,
                    o.isDA ? nfree : -llh, llh, diff);
            fflush(g_log);
            if (o.log_progress) {
                tr_temp.push_back(temp);
                tr_llh.push_back(llh);
                if (o.isDA)
                    tr_free.push_back(nfree);
            }
            if ((o.checkpointing && (nloop % o.period) == 0) || g_force_checkpoint) {
                // dagtm/dagtm.cxx:1609-1687
                char name[4096];
                snprintf(name, sizeof(name), "%s%d.h5", o.prefix.c_str(), nloop);
                check(dgtm_get_Y(ctx, Y.data(), D), "dgtm_get_Y");
                h5lite::Writer w;
                w.add_f64(o.dX, {(uint64_t) K, (uint64_t) L}, X.data());
                w.add_f64(o.dFI, {(uint64_t) K, (uint64_t) M + 1}, FI.data());
                w.add_f64(o.dY, {(uint64_t) K, (uint64_t) D}, Y.data());
                w.add_scalar_f64(o.dbeta, beta);
                w.add_scalar_f64(o.dtemp, temp);
                w.add_scalar_i32(o.diter, nloop);
                w.add_scalar_i32(o.dseed, (int32_t) seed);
                w.add_scalar_f64(o.dqual, qual);
                if (!w.write(name, err))
                    die("%s", err.c_str());
                if (g_force_checkpoint) {
                    fprintf(stderr, "dagtm: forced checkpoint %s written\n", name);
                    dgtm_ctx_destroy(ctx);
                    return 0;
                }
            }
            if (fabs(diff) < o.eps)
                break;
            if (nloop > QUEUE) {
                double s0 = 0;
                for (double v : queue)
                    s0 += v;
                const double avg_old = s0 / QUEUE;
                queue[qnext] = qual;
                qnext = (qnext + 1) % QUEUE;
                double s1 = 0;
                for (double v : queue)
                    s1 += v;
                if (fabs(s1 / QUEUE - avg_old) < o.eps) {
                    fprintf(stderr, "dagtm: average of %d iterations has converged\n", QUEUE);
                    break;
                }
            }
            check(dgtm_mstep(ctx, W.data(), D, nullptr, D, &beta), "dgtm_mstep");
            have_W = true;
            if (o.schedule == 2 || o.hda) {
                // AUTO and HDA weigh centres by the G of the last M-step
                G_last.resize(K);
                check(dgtm_get_stats(ctx, G_last.data(), nullptr, D), "dgtm_get_stats");
            }
            stats_current = false;
            if (maxloop && nloop >= maxloop) {
                isLast = true;
                break;
            }
        }
        if (o.isDA && !isLast) {
            if (o.schedule == 1) {
                temp -= o.delta;
            } else if (o.schedule == 2) {
                // dagtm/dagtm.cxx:1919-1934: the next critical temperature, with
                // the G of the last M-step as the per-centre weights
                double ct = 0.0;
                check(dgtm_next_ctemp(ctx, temp, beta, o.eps,
                                      G_last.empty() ? nullptr : G_last.data(), &ct),
                      "dgtm_next_ctemp");
                if (ct >= temp)
                    ct = temp * o.alpha;  // no valid next critical temperature
                temp = ct;
            } else {
                if (o.hda && K < o.Kmax)
                    hda_step(qual_before_temp);
                temp *= o.alpha;
            }
        } else {
            break;
        }
    } while (!isLast);
    const clock_t en_time = times(&en_cpu);
    check(dgtm_get_Y(ctx, Y.data(), D), "dgtm_get_Y");
    if (!have_W)
        W.clear();

    // ---- summary (dagtm/dagtm.cxx:2213-2283)
    fprintf(g_log, "Done.\n");
    fprintf(g_log, "==================== SUMMARY ====================\n");
    fprintf(g_log, "%20s = %s\n", "Data filename", o.in.c_str());
    fprintf(g_log, "%20s = %dx%d\n", "Compute Grid", 1, 1);
    fprintf(g_log, "%20s = %d\n", "N", N);
    fprintf(g_log, "%20s = %d\n", "D", D);
    fprintf(g_log, "%20s = %d\n", "K", K);
    fprintf(g_log, "%20s = %d\n", "L", L);
    fprintf(g_log, "%20s = %d\n", "M", M);
    fprintf(g_log, "%20s = %ld\n", "SEED", (long) seed);
    fprintf(g_log, "%20s = %.10g\n", "Max. Qual", qual);
    fprintf(g_log, "%20s = %s\n", "Grid Type", "SWEEP");
    if (o.isDA) {
        fprintf(g_log, "%20s = %.10g\n", "Start Temp", start_temp);
        fprintf(g_log, "%20s = %.10g\n", "1st Critical Temp", first_ctemp);
        if (o.schedule == 2) {
            fprintf(g_log, "%20s = %s\n", "Cooling Schedule", "AUTO");
        } else if (o.schedule == 0) {
            fprintf(g_log, "%20s = %s\n", "Cooling Schedule", "EXP");
            fprintf(g_log, "%20s = %g\n", "alpha", o.alpha);
            if (o.hda)
                fprintf(g_log, "%20s = %d (K = %d)\n", "HDA expansions", nexpanded, K);
        } else {
            fprintf(g_log, "%20s = %s\n", "Cooling Schedule", "LINEAR");
            fprintf(g_log, "%20s = %g\n", "delta", o.delta);
        }
    }
    fprintf(g_log, "%20s = %d\n", "Num. of Iterations", nloop);
    fprintf(g_log, "-------------------------------------------------\n");
    fprintf(g_log, "%20s = %.03f\n", "Real Time(s)", (double) (en_time - st_time) / clk_tck);
    fprintf(g_log, "%20s = %.03f\n", "User Time(s)",
            (double) (en_cpu.tms_utime - st_cpu.tms_utime) / clk_tck);
    fprintf(g_log, "%20s = %.03f\n", "System Time(s)",
            (double) (en_cpu.tms_stime - st_cpu.tms_stime) / clk_tck);
    fprintf(g_log, "=================================================\n");
    fflush(g_log);

    // ---- output (dagtm/dagtm.cxx:2342-2552): the MAP needs responsibilities
    // of the final centres.  After a maxloop break the reference reuses the R
    // that dagtm_mpi_beta multiplied by the new distances (comm/mpicomm.c:288):
    // with -J this driver writes that R o D too; by default it runs one more
    // E-step on the final centres instead.
    if (!o.out.empty()) {
        const bool rd = o.rd_output && !stats_current;
        if (!stats_current && !rd)
            check(dgtm_estep(ctx, beta, o.isDA, temp, &llh, &nfree), "dgtm_estep");
        std::vector<double> Mout((size_t) N * L);
        if (rd)
            check(dgtm_map_rd(ctx, X.data(), L, Mout.data(), L), "dgtm_map_rd");
        else
            check(dgtm_map(ctx, X.data(), L, Mout.data(), L), "dgtm_map");
        h5lite::Writer w = write_output(Mout, qual, o.save_R, rd);
        for (const Snap &sn : snaps)
            w.add_f64(sn.name, sn.dims, sn.v.data());
        if (o.log_progress) {
            w.add_f64("Temp", {(uint64_t) tr_temp.size()}, tr_temp.data());
            w.add_f64("LLH", {(uint64_t) tr_llh.size()}, tr_llh.data());
            if (o.isDA)
                w.add_f64("NFree", {(uint64_t) tr_free.size()}, tr_free.data());
        }
        if (!w.write(o.out, err))
            die("%s", err.c_str());
    }
    dgtm_ctx_destroy(ctx);
    if (g_log != stdout)
        fclose(g_log);
    return 0;
}
