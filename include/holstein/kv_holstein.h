/* Drop-in C++ layer: the class names and calls of the reference's holstein/
 * headers that its drivers use (src/kln-tdvp.cpp:7, 73-78), implemented on
 * the C ABI of libkvgpu (include/kvgpu.h).  Header-only; link with -lkvgpu.
 *
 * Placed as the `holstein/` directory next to a driver's `src/`, it lets
 * `#include "../holstein/tdvp.h"` resolve here, so the driver compiles
 * unchanged and its sweeps run on the GPU.
 *
 * Also provided: State::canonicalize and Operator::join (on the device), the
 * scalar products and the direct sums State += / Operator +=
 * (holstein/state.h:54-85, holstein/operator.h:54-70).
 * Reference behaviour kept: the binary .mps / .mpo formats
 * (holstein/state.h:107-157, holstein/operator.h:117-143), parse_stage
 * (holstein/tdvp.h:19-32), the TDVP constructor's arguments
 * (holstein/tdvp.h:60-76) and total_start's stages with a checkpoint
 * State/T-<sweep>.mps after every sweep (holstein/tdvp.h:297-385), including
 * the SA-1TDVP stage: the two-site sweeps append the SVS log
 * (holstein/svd.h:390-402), the stage runs `nls.py` from PATH to fit it and
 * reads the widths it writes to `beta`, as the reference does (this
 * package's kylin-v_gb300/sa_fit.py restates that fit and can be installed
 * under that name); errors print a message and exit(1) as the reference does.
 * Differences: after the global-Krylov stage (r[0] > 0) the sweep
 * environments are rebuilt from the new state (the reference keeps the ones
 * built before that stage); the SA stage's draws come from one seed
 * (std::random_device, or KV_SA_SEED when set) instead of a fresh
 * random_device per draw group; the timer table lists device milliseconds
 * per module.  Environment: KV_PRECISION=mixed selects the mixed-precision
 * path (default FP64), KV_DEVICE the GPU (default 0). */
#ifndef KV_HOLSTEIN_DROPIN_H
#define KV_HOLSTEIN_DROPIN_H

#include <sys/stat.h>

#include <array>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "../kvgpu.h"

namespace KylinVib {
using namespace std;
typedef int INT;
typedef complex<double> Complex;

namespace Holstein {
namespace detail {

inline void check(int rc, const char *what) {
    if (rc != KV_OK) {
        cout << what << " failed: " << kv_last_error() << endl;
        exit(1);
    }
}

inline void ensure_init() {
    static bool done = false;
    if (done) return;
    const char *d = getenv("KV_DEVICE");
    check(kv_init(d ? atoi(d) : 0), "kv_init");
    done = true;
}

inline int precision() {
    const char *p = getenv("KV_PRECISION");
    return (p && strcmp(p, "mixed") == 0) ? KV_MIXED_TF32 : KV_FP64;
}

}  // namespace detail

// A block-sparse tensor of rank R on the host: blocks in file order, each a
// dense row-major complex128 array with its shape and leg charges.
template <int R>
struct HostTensor {
    array<INT, R> dirs{};
    vector<array<INT, R>> shape, qn;
    vector<vector<Complex>> data;

    INT num_blocks() const { return (INT)shape.size(); }

    void read_blocks(ifstream &ifs, INT nb) {
        for (INT j = 0; j < nb; ++j) {
            array<INT, R> sp, q;
            ifs.read(reinterpret_cast<char *>(sp.data()), sizeof(INT) * R);
            ifs.read(reinterpret_cast<char *>(q.data()), sizeof(INT) * R);
            size_t n = 1;
            for (INT s : sp) n *= (size_t)s;
            vector<Complex> v(n);
            ifs.read(reinterpret_cast<char *>(v.data()), sizeof(Complex) * n);
            shape.push_back(sp);
            qn.push_back(q);
            data.push_back(move(v));
        }
    }

    void write_blocks(ofstream &ofs) const {
        INT nb = num_blocks();
        ofs.write(reinterpret_cast<const char *>(&nb), sizeof(INT));
        for (INT j = 0; j < nb; ++j) {
            ofs.write(reinterpret_cast<const char *>(shape[j].data()), sizeof(INT) * R);
            ofs.write(reinterpret_cast<const char *>(qn[j].data()), sizeof(INT) * R);
            ofs.write(reinterpret_cast<const char *>(data[j].data()), sizeof(Complex) * data[j].size());
        }
    }

    // a device copy (caller frees with kv_tensor_free)
    kv_tensor upload() const {
        vector<int> sh, q;
        vector<double> d;
        for (INT j = 0; j < num_blocks(); ++j) {
            sh.insert(sh.end(), shape[j].begin(), shape[j].end());
            q.insert(q.end(), qn[j].begin(), qn[j].end());
            const double *p = reinterpret_cast<const double *>(data[j].data());
            d.insert(d.end(), p, p + 2 * data[j].size());
        }
        kv_tensor t = nullptr;
        detail::check(kv_tensor_create(R, dirs.data(), num_blocks(), sh.data(), q.data(), d.data(), &t),
                      "kv_tensor_create");
        return t;
    }

    static HostTensor download(kv_tensor t) {
        int rank = 0, nb = 0;
        long long ne = 0;
        detail::check(kv_tensor_info(t, &rank, &nb, &ne), "kv_tensor_info");
        if (rank != R) {
            cout << "unexpected tensor rank " << rank << endl;
            exit(1);
        }
        vector<int> sh((size_t)nb * R), q((size_t)nb * R);
        vector<double> d(2 * (size_t)ne);
        HostTensor h;
        detail::check(kv_tensor_download(t, h.dirs.data(), sh.data(), q.data(), d.data()), "kv_tensor_download");
        size_t off = 0;
        for (int j = 0; j < nb; ++j) {
            array<INT, R> s, c;
            size_t n = 1;
            for (int i = 0; i < R; ++i) {
                s[i] = sh[(size_t)j * R + i];
                c[i] = q[(size_t)j * R + i];
                n *= (size_t)s[i];
            }
            vector<Complex> v(n);
            for (size_t k = 0; k < n; ++k) v[k] = Complex(d[2 * (off + k)], d[2 * (off + k) + 1]);
            off += n;
            h.shape.push_back(s);
            h.qn.push_back(c);
            h.data.push_back(move(v));
        }
        return h;
    }
};

namespace detail {

// b added into a as a direct sum along the legs `axes` (holstein/tensor.h
// stack, :263-320): on each such leg a charge sector's dimension becomes the
// sum of the two tensors' dimensions, a's entries first and b's after them;
// every block is zero-padded to its combined shape, then blocks of equal
// shape and charges are added.  Host-side, like the reference's.
template <int R>
void stack_into(HostTensor<R> &a, const HostTensor<R> &b, const vector<int> &axes) {
    auto legs = [](const HostTensor<R> &t) {
        array<map<INT, INT>, R> l;
        for (INT j = 0; j < t.num_blocks(); ++j)
            for (int i = 0; i < R; ++i) l[i][t.qn[j][i]] = t.shape[j][i];
        return l;
    };
    const array<map<INT, INT>, R> lb = legs(b);
    array<map<INT, INT>, R> comb = legs(a);
    for (int ax : axes)
        for (const auto &kv : lb[ax]) comb[ax][kv.first] += kv.second;
    // src (shape sp) placed at offset pos of a zero block of shape full, row-major
    auto embed = [](const vector<Complex> &src, const array<INT, R> &sp, const array<INT, R> &full,
                    const array<INT, R> &pos) {
        size_t n = 1;
        for (INT x : full) n *= (size_t)x;
        vector<Complex> out(n);
        for (size_t e = 0; e < src.size(); ++e) {
            size_t rem = e, dst = 0, stride = 1;
            array<size_t, R> idx{};
            for (int i = R - 1; i >= 0; --i) {
                idx[i] = rem % (size_t)sp[i];
                rem /= (size_t)sp[i];
            }
            for (int i = R - 1; i >= 0; --i) {
                dst += (idx[i] + (size_t)pos[i]) * stride;
                stride *= (size_t)full[i];
            }
            out[dst] = src[e];
        }
        return out;
    };
    for (INT j = 0; j < a.num_blocks(); ++j) {
        array<INT, R> full = a.shape[j], pos{};
        for (int ax : axes) full[ax] = comb[ax][a.qn[j][ax]];
        if (full != a.shape[j]) {
            a.data[j] = embed(a.data[j], a.shape[j], full, pos);
            a.shape[j] = full;
        }
    }
    for (INT j = 0; j < b.num_blocks(); ++j) {
        array<INT, R> full = b.shape[j], pos{};
        for (int ax : axes) {
            full[ax] = comb[ax][b.qn[j][ax]];
            pos[ax] = full[ax] - b.shape[j][ax];
        }
        vector<Complex> blk = full == b.shape[j] ? b.data[j] : embed(b.data[j], b.shape[j], full, pos);
        bool added = false;
        for (INT k = 0; k < a.num_blocks() && !added; ++k)
            if (a.shape[k] == full && a.qn[k] == b.qn[j]) {
                for (size_t e = 0; e < blk.size(); ++e) a.data[k][e] += blk[e];
                added = true;
            }
        if (!added) {
            a.shape.push_back(full);
            a.qn.push_back(b.qn[j]);
            a.data.push_back(move(blk));
        }
    }
}

}  // namespace detail

// Holstein::State: an MPS, legs (left bond, phys, right bond), dirs {1, 1, -1}
class State {
  public:
    State() = default;
    explicit State(INT ns) : tt_(ns) {
        for (auto &t : tt_) t.dirs = {1, 1, -1};
    }

    static State load(ifstream &ifs) {
        INT label = 0, ns = 0;
        ifs.read(reinterpret_cast<char *>(&label), sizeof(INT));
        if (label != 111) {
            cout << "Illegal MPS file!" << endl;
            exit(1);
        }
        ifs.read(reinterpret_cast<char *>(&ns), sizeof(INT));
        State res(ns);
        for (INT i = 0; i < ns; ++i) {
            INT nb = 0;
            ifs.read(reinterpret_cast<char *>(&nb), sizeof(INT));
            res.tt_[i].read_blocks(ifs, nb);
        }
        ifs.close();
        return res;
    }

    void save(ofstream &ofs) const {
        INT label = 111, ns = nsite();
        ofs.write(reinterpret_cast<const char *>(&label), sizeof(INT));
        ofs.write(reinterpret_cast<const char *>(&ns), sizeof(INT));
        for (const auto &t : tt_) t.write_blocks(ofs);
        ofs << endl;
        ofs.close();
    }

    INT nsite() const { return (INT)tt_.size(); }
    HostTensor<3> &operator[](INT i) { return tt_[i]; }
    const HostTensor<3> &at(INT i) const { return tt_[i]; }

    // direct sum: the MPS of this + r, bond dimensions added
    // (holstein/state.h:54-64)
    State &operator+=(const State &r) {
        const INT ns = nsite();
        if (r.nsite() != ns || ns < 2) {
            cout << "State += : the states differ in length" << endl;
            exit(1);
        }
        detail::stack_into(tt_[0], r.tt_[0], {2});
        for (INT i = 1; i < ns - 1; ++i) detail::stack_into(tt_[i], r.tt_[i], {0, 2});
        detail::stack_into(tt_[ns - 1], r.tt_[ns - 1], {0});
        return *this;
    }

    // the scalar multiplies site 0 (holstein/state.h:66-85)
    State &operator*=(double val) {
        for (auto &b : tt_.at(0).data)
            for (auto &x : b) x *= val;
        return *this;
    }
    State operator*(const Complex &val) const {
        State res(*this);
        for (auto &b : res.tt_.at(0).data)
            for (auto &x : b) x *= val;
        return res;
    }
    State operator*(double val) const { return (*this) * Complex(val, 0.0); }

    // an L->R then an R->L SVD sweep on the device, the orthogonality centre
    // left on site 0 (holstein/state.h:166-185)
    void canonicalize(double tolS = 0.0, INT mD = 1000) {
        detail::ensure_init();
        const INT ns = nsite();
        vector<kv_tensor> in(ns), out(ns, nullptr);
        for (INT i = 0; i < ns; ++i) in[i] = tt_[i].upload();
        const int rc = kv_canonicalize(ns, in.data(), tolS, mD, detail::precision(), out.data());
        for (auto t : in) kv_tensor_free(t);
        detail::check(rc, "canonicalize");
        for (INT i = 0; i < ns; ++i) {
            tt_[i] = HostTensor<3>::download(out[i]);
            kv_tensor_free(out[i]);
        }
    }

    // largest right bond dimension and its position (holstein/state.h:187-200)
    void max_bond() const {
        INT mb = 0, mbp = 0;
        for (INT i = 0; i + 1 < nsite(); ++i) {
            // sum of the distinct (charge, dimension) pairs of leg 2
            vector<pair<INT, INT>> seen;
            INT cur = 0;
            for (INT j = 0; j < tt_[i].num_blocks(); ++j) {
                pair<INT, INT> k{tt_[i].qn[j][2], tt_[i].shape[j][2]};
                bool dup = false;
                for (auto &x : seen) dup = dup || x.first == k.first;
                if (!dup) {
                    seen.push_back(k);
                    cur += k.second;
                }
            }
            if (mbp < cur) {
                mb = i;
                mbp = cur;
            }
        }
        cout << "Max bond dimension = " << mbp << " on bond " << mb << "-" << mb + 1 << endl;
    }

  private:
    vector<HostTensor<3>> tt_;
};

// Holstein::Operator: an MPO, legs (phys_out, left bond, phys_in, right bond), dirs {1, 1, -1, -1}
class Operator {
  public:
    Operator() = default;
    explicit Operator(INT ns) : tt_(ns) {
        for (auto &t : tt_) t.dirs = {1, 1, -1, -1};
    }

    static Operator load(ifstream &ifs) {
        INT label = 0, ns = 0;
        ifs.read(reinterpret_cast<char *>(&label), sizeof(INT));
        if (label != 112) {
            cout << "Illegal MPO file!" << endl;
            exit(1);
        }
        ifs.read(reinterpret_cast<char *>(&ns), sizeof(INT));
        Operator res(ns);
        for (INT i = 0; i < ns; ++i) {
            INT nb = 0;
            ifs.read(reinterpret_cast<char *>(&nb), sizeof(INT));
            res.tt_[i].read_blocks(ifs, nb);
        }
        return res;
    }

    INT nsite() const { return (INT)tt_.size(); }
    HostTensor<4> &operator[](INT i) { return tt_[i]; }
    const HostTensor<4> &at(INT i) const { return tt_[i]; }

    // direct sum: the MPO of this + r, MPO bond dimensions added
    // (holstein/operator.h:54-64)
    Operator &operator+=(const Operator &r) {
        const INT ns = nsite();
        if (r.nsite() != ns || ns < 2) {
            cout << "Operator += : the operators differ in length" << endl;
            exit(1);
        }
        detail::stack_into(tt_[0], r.tt_[0], {3});
        for (INT i = 1; i < ns - 1; ++i) detail::stack_into(tt_[i], r.tt_[i], {1, 3});
        detail::stack_into(tt_[ns - 1], r.tt_[ns - 1], {1});
        return *this;
    }

    // the scalar multiplies site 0 (holstein/operator.h:66-70)
    Operator &operator*=(double val) {
        for (auto &b : tt_.at(0).data)
            for (auto &x : b) x *= val;
        return *this;
    }

    // <s1|this|s2> on the device (holstein/operator.h:178-198)
    Complex join(const State &s1, const State &s2) const {
        detail::ensure_init();
        const INT ns = nsite();
        if (s1.nsite() != ns || s2.nsite() != ns) {
            cout << "join: the states and the operator differ in length" << endl;
            exit(1);
        }
        vector<kv_tensor> a(ns), w(ns), b(ns);
        for (INT i = 0; i < ns; ++i) {
            a[i] = s1.at(i).upload();
            w[i] = tt_[i].upload();
            b[i] = s2.at(i).upload();
        }
        double re = 0.0, im = 0.0;
        const int rc = kv_expectation(ns, a.data(), w.data(), b.data(), &re, &im);
        for (INT i = 0; i < ns; ++i) {
            kv_tensor_free(a[i]);
            kv_tensor_free(w[i]);
            kv_tensor_free(b[i]);
        }
        detail::check(rc, "join");
        return Complex(re, im);
    }

  private:
    vector<HostTensor<4>> tt_;
};

// "[nK,n2,nsa,n1]" -> {nK, n2, nsa, n1} (holstein/tdvp.h:19-32)
inline array<INT, 4> parse_stage(const string &s) {
    array<INT, 4> r{};
    stringstream ss(s.substr(1, s.size() - 1));
    string tmp;
    for (INT i = 0; i < 4; ++i) {
        getline(ss, tmp, ',');
        r[i] = (INT)stol(tmp);
    }
    return r;
}

// Holstein::TDVP on the device (holstein/tdvp.h:34-385)
class TDVP {
  public:
    TDVP(State &MPS, Operator &MPO, double tolSVD, double tolExp, INT maxDim, INT maxIter, double timeStep)
        : mps_(move(MPS)), ham_(move(MPO)) {
        detail::ensure_init();
        const INT ns = mps_.nsite();
        vector<kv_tensor> m, w;
        for (INT i = 0; i < ns; ++i) {
            m.push_back(mps_.at(i).upload());
            w.push_back(ham_.at(i).upload());
        }
        detail::check(kv_tdvp_create(ns, m.data(), w.data(), tolSVD, tolExp, maxDim, maxIter, timeStep,
                                     detail::precision(), &s_),
                      "kv_tdvp_create");
        for (auto t : m) kv_tensor_free(t);
        for (auto t : w) kv_tensor_free(t);
        cout << "Krylov: tolerance " << tolExp << ", max iterations " << maxIter << ", time step " << timeStep
             << "\nSVD: cutoff " << tolSVD << ", max bond " << maxDim
             << (detail::precision() == KV_FP64 ? "\nprecision: FP64" : "\nprecision: mixed") << endl;
        ofstream ofs("SVS");
        ofs << "Total Site = " << ns << endl;
        int nr = 0;
        long long nv = 0;
        detail::check(kv_tdvp_svs(s_, &nr, &nv, nullptr, nullptr), "kv_tdvp_svs");  // starts the record
    }
    TDVP(const TDVP &) = delete;
    TDVP &operator=(const TDVP &) = delete;
    ~TDVP() {
        if (s_) kv_tdvp_free(s_);
    }

    void one_site() { sweep(1); }
    void two_site() {
        sweep(2);
        append_svs();
    }
    // TDVP::sa_site (holstein/tdvp.h:230-294)
    void sa_site(vector<double> &betaSet) {
        unsigned long long seed = std::random_device{}();
        if (const char *e = getenv("KV_SA_SEED")) seed = strtoull(e, nullptr, 10);
        if (!sa_set_) {
            detail::check(kv_tdvp_set_sa(s_, betaSet.data(), (int)betaSet.size(), seed, nullptr), "kv_tdvp_set_sa");
            sa_set_ = true;
        }
        sweep(3);
    }
    const State &state() const { return mps_; }

    void total_start(const array<INT, 4> &r) {
        INT swp = 0;
        cout << "\n ---------------- Start Krylov stage ----------------" << endl;
        for (; swp < r[0]; ++swp) {
            sweep(0);
            checkpoint(swp);
        }
        cout << "\n ---------------- Start 2TDVP stage ----------------" << endl;
        for (; swp < r[0] + r[1]; ++swp) {
            cout << "\nSweep " << swp + 1 << ":" << endl;
            two_site();
            checkpoint(swp);
        }
        if (r[2] != 0) {
            vector<double> betaSet;
            int ifos = system("nls.py");
            (void)ifos;
            cout << "Fitting OK!" << endl;
            ifstream ifsBeta("beta");
            if (!ifsBeta.is_open()) cout << "Fail to open beta file" << endl;
            string tmp;
            while (getline(ifsBeta, tmp))
                if (tmp.size() > 3) betaSet.push_back(1.0 / stod(tmp));
            cout << "Read betas OK!" << endl;
            if ((INT)betaSet.size() < mps_.nsite() - 1) {
                cout << "The beta file holds " << betaSet.size() << " widths; the SA-1TDVP stage needs one per bond."
                     << endl;
                exit(1);
            }
            cout << "\n ---------------- Start SA-1TDVP stage -------------" << endl;
            for (; swp < r[0] + r[1] + r[2]; ++swp) {
                cout << "\nSweep " << swp + 1 << ":" << endl;
                sa_site(betaSet);
                checkpoint(swp);
            }
        }
        cout << "\n ---------------- Start 1TDVP stage ----------------" << endl;
        for (; swp < r[0] + r[1] + r[2] + r[3]; ++swp) {
            cout << "\nSweep " << swp + 1 << ":" << endl;
            one_site();
            checkpoint(swp);
        }
        static const char *names[6] = {"Evl-0", "Evl-1", "Evl-2", "SVD", "Update", "Sweep"};
        cout << "\n Module        device ms" << endl;
        for (int i = 0; i < 6; ++i) cout << " " << names[i] << "\t" << total_ms_[i] << endl;
    }

  private:
    void sweep(int mode) {
        detail::check(kv_tdvp_sweep(s_, mode), "kv_tdvp_sweep");
        if (mode != 0) {  // the module timings cover the TDVP sweeps
            double ms[6], sw, fl, fg;
            detail::check(kv_tdvp_stats(s_, ms, &sw, &fl, &fg), "kv_tdvp_stats");
            for (int i = 0; i < 6; ++i) total_ms_[i] += ms[i];
        }
        for (INT i = 0; i < mps_.nsite(); ++i) {
            kv_tensor t = nullptr;
            detail::check(kv_tdvp_site(s_, i, &t), "kv_tdvp_site");
            mps_[i] = HostTensor<3>::download(t);
            kv_tensor_free(t);
        }
    }

    // the two-site splits' records of the SVS log, in svd_impl's format
    // (holstein/svd.h:390-402): the kept count, then log10(s_i s_{i-2} / s_{i-1}^2)
    void append_svs() {
        int nr = 0;
        long long nv = 0;
        detail::check(kv_tdvp_svs(s_, &nr, &nv, nullptr, nullptr), "kv_tdvp_svs");
        vector<int> counts(nr > 0 ? nr : 1);
        vector<double> vals(nv > 0 ? nv : 1);
        detail::check(kv_tdvp_svs(s_, nullptr, nullptr, counts.data(), vals.data()), "kv_tdvp_svs");
        ofstream ofs("SVS", ofstream::app);
        long long k = 0;
        for (int r = 0; r < nr; ++r) {
            const double *v = vals.data() + k;
            ofs << counts[r] << endl;
            for (int i = 2; i < counts[r]; ++i)
                ofs << std::left << setw(20) << std::scientific << setprecision(11)
                    << log10(v[i] * v[i - 2] / pow(v[i - 1], 2.0)) << endl;
            k += counts[r];
        }
    }

    void checkpoint(INT swp) {
        mps_.max_bond();
        mkdir("State", 0755);
        ofstream ofs("State/T-" + to_string(swp) + ".mps");
        mps_.save(ofs);
    }

    State mps_;
    Operator ham_;
    kv_tdvp s_ = nullptr;
    bool sa_set_ = false;
    double total_ms_[6] = {};
};

}  // namespace Holstein
}  // namespace KylinVib

#endif
