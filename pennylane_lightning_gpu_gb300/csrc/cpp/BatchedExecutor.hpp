// BatchedExecutor<P>: many independent parameterised circuits in one
// persistent, CUDA-graph-captured launch (lgpu_batch_* in lgpu.h).
//
// Host side: each circuit's operations are lowered with the same dispatcher
// as StateVectorCudaManaged, fused into blocks whose targets fit a
// shared-memory tile (a circuit of n <= kmax qubits is one block holding the
// whole state), and flattened into device records.  Parametric gates keep a
// parameter index, so run(params) only copies the new parameter vector; the
// graph [params H2D, matrix build, counter reset, persistent kernel, results
// D2H] is captured once at prepare() and replayed for every run().
#pragma once

#include <algorithm>
#include <atomic>
#include <cstring>
#include <exception>
#include <memory>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "GateLowering.hpp"
#include "cuda_helpers.hpp"

namespace Pennylane {

template <class Precision> class BatchedExecutor {
  public:
    using cd = std::complex<double>;
    static constexpr lgpu_dtype_t dt = cuUtil::dtype_of<Precision>();

    struct PTerm {
        double coeff;
        std::string word;
        std::vector<size_t> wires;
    };

    explicit BatchedExecutor(int kmax = 0, int threads = 256, int grid = 0)
        : kmax_(kmax > 0 ? kmax : (std::is_same_v<Precision, double> ? 13 : 14)), threads_(threads), grid_(grid) {
        PL_ABORT_IF(kmax_ > (std::is_same_v<Precision, double> ? 13 : 14) || kmax_ < 6, "kmax out of range");
        PL_LGPU_IS_SUCCESS(lgpu_stream_create(&stream_));
    }
    ~BatchedExecutor() {
        release();
        if (stream_) lgpu_stream_destroy(stream_);
    }
    BatchedExecutor(const BatchedExecutor &) = delete;
    BatchedExecutor &operator=(const BatchedExecutor &) = delete;

    // Add a circuit; returns its index.  params[i] are the op's parameters;
    // those of the parametric gates (RX, RY, RZ, their controlled forms,
    // PhaseShift, ControlledPhaseShift, Rot, CRot, IsingXX/YY/ZZ) are appended
    // to the executor's parameter vector in op order (the circuit's first one
    // is at paramOffset()); the others are built into fixed matrices.
    size_t addCircuit(size_t n, const std::vector<std::string> &names, const std::vector<std::vector<size_t>> &wires,
                      const std::vector<std::vector<double>> &params, const std::vector<bool> &inverses,
                      const std::vector<PTerm> &observable) {
        PL_ABORT_IF(prepared_, "addCircuit after prepare()");
        auto shape = makeShape(n, names, wires, params, inverses, observable, params_);
        const size_t off = params_.size() - shape->nparams;
        circuits_.push_back(Circuit{std::move(shape), off});
        return circuits_.size() - 1;
    }

    // A circuit structure shared by many parameter sets (a template): it is
    // lowered and fused once.  `params` gives the operations' parameters; those
    // of the parametric gates are placeholders that every instance replaces
    // (templateNumParams() of them, in op order), the others are fixed.
    size_t addTemplate(size_t n, const std::vector<std::string> &names, const std::vector<std::vector<size_t>> &wires,
                       const std::vector<std::vector<double>> &params, const std::vector<bool> &inverses,
                       const std::vector<PTerm> &observable) {
        PL_ABORT_IF(prepared_, "addTemplate after prepare()");
        std::vector<double> placeholders;
        templates_.push_back(makeShape(n, names, wires, params, inverses, observable, placeholders));
        return templates_.size() - 1;
    }
    size_t templateNumParams(size_t tid) const { return templates_.at(tid)->nparams; }

    // `count` circuits of template `tid`, instance i taking the parameters
    // params[i * P .. (i + 1) * P) with P = templateNumParams(tid); returns the
    // index of the first new circuit.
    size_t addInstances(size_t tid, const double *params, size_t count) {
        PL_ABORT_IF(prepared_, "addInstances after prepare()");
        PL_ABORT_IF(tid >= templates_.size(), "unknown template");
        const auto &shape = templates_[tid];
        const size_t P = shape->nparams;
        const size_t first = circuits_.size();
        params_.reserve(params_.size() + count * P);
        circuits_.reserve(circuits_.size() + count);
        for (size_t i = 0; i < count; i++) {
            circuits_.push_back(Circuit{shape, params_.size()});
            params_.insert(params_.end(), params + i * P, params + (i + 1) * P);
        }
        return first;
    }

    size_t paramOffset(size_t circuit) const { return circuits_.at(circuit).param_off; }
    size_t numParams() const { return params_.size(); }
    size_t numCircuits() const { return circuits_.size(); }
    int kmax() const { return kmax_; }
    // tile bits of circuits above kmax qubits (a 3-stage ring of 64 KB tiles)
    int klarge() const { return std::is_same_v<Precision, double> ? 12 : 13; }

    // capture = true: one eager run (sets kernel attributes, validates), then
    // the graph is captured and every run() replays it.  capture = false: no
    // run and no graph; every run() enqueues the steps directly (for a batch
    // that runs once, e.g. one micro-batch of a server).
    void prepare(bool capture = true) {
        PL_ABORT_IF(prepared_, "prepare() called twice");
        PL_ABORT_IF(circuits_.empty(), "no circuits");
        std::vector<lgpu_bcircuit_t> hc;
        std::vector<lgpu_bblock_t> hb;
        std::vector<lgpu_bgate_t> hg;
        std::vector<lgpu_bterm_t> ht;
        std::vector<double> pool;
        std::vector<double> cost(circuits_.size());
        size_t max_big = 0;
        planShapes();
        for (size_t ci = 0; ci < circuits_.size(); ci++) {
            const Shape &c = *circuits_[ci].shape;
            const size_t param_off = circuits_[ci].param_off;
            lgpu_bcircuit_t rec{};
            rec.n = uint32_t(c.n);
            rec.block_off = uint32_t(hb.size());
            rec.out = uint32_t(ci);
            if (int(c.n) > kmax_) max_big = std::max(max_big, c.n);
            // blocks: [(tile bits, gate indices)], planned once per shape
            const auto &blocks = planBlocks(*circuits_[ci].shape);
            double work = 0;
            for (const auto &blk : blocks) {
                lgpu_bblock_t b{};
                b.k = uint8_t(blk.first.size());
                int m = 0;
                while (m < int(blk.first.size()) && blk.first[size_t(m)] == m) m++;
                b.m = uint8_t(m);
                PL_ABORT_IF(b.k - b.m > 6, "tile has more than 6 high bits");
                for (size_t q = 0; q < blk.first.size(); q++) b.bits[q] = uint8_t(blk.first[q]);
                b.gate_off = uint32_t(hg.size());
                std::vector<int> pos(c.n, -1);
                for (size_t q = 0; q < blk.first.size(); q++) pos[size_t(blk.first[q])] = int(q);
                // runs of uncontrolled 1-target gates on one bit become one
                // chain head (its matrix is their product, built on the
                // device) followed by the folded gates, which the kernel skips
                const auto &gl = blk.second;
                auto single = [&](size_t gi) {
                    const Op &o = c.ops[gi];
                    return o.tgts.size() == 1 && o.ctrls.empty() && o.kind < 5;
                };
                for (size_t i = 0; i < gl.size();) {
                    size_t j = i + 1;
                    if (single(gl[i]))
                        while (j < gl.size() && j - i < kMaxChain && single(gl[j]) &&
                               c.ops[gl[j]].tgts[0] == c.ops[gl[i]].tgts[0])
                            j++;
                    if (j - i >= 2) {
                        lgpu_bgate_t head{};
                        head.kind = 0;  // dense 1-target
                        head.q0 = uint8_t(pos[size_t(c.ops[gl[i]].tgts[0])]);
                        head.q1 = uint8_t(j - i);
                        head.flags = 2u;
                        head.param = -1;
                        head.mat = uint32_t(pool.size());
                        pool.resize(pool.size() + 16, 0.0);
                        hg.push_back(head);
                        for (size_t t = i; t < j; t++) {
                            lgpu_bgate_t g = record(c.ops[gl[t]], pos, param_off, pool);
                            g.kind = 7;  // folded into the head
                            hg.push_back(g);
                        }
                    } else {
                        hg.push_back(record(c.ops[gl[i]], pos, param_off, pool));
                    }
                    i = j;
                }
                b.gate_cnt = uint32_t(hg.size() - b.gate_off);
                hb.push_back(b);
                work += double(blk.second.size() + 2) * std::ldexp(1.0, int(c.n));
            }
            rec.block_cnt = uint32_t(blocks.size());
            // observable terms, flips in tile positions of the last block
            rec.obs_off = uint32_t(ht.size());
            const auto &last = blocks.back().first;
            std::vector<int> pos(c.n, -1);
            for (size_t q = 0; q < last.size(); q++) pos[size_t(last[q])] = int(q);
            for (const auto &t : c.obs) {
                lgpu_bterm_t term{};
                int ny = 0;
                for (size_t k = 0; k < t.word.size(); k++) {
                    const int b = Engine::bit_of(c.n, t.wires[k]);
                    const char ch = t.word[k];
                    if (ch == 'X' || ch == 'Y') term.tflip |= uint64_t(1) << pos[size_t(b)];
                    if (ch == 'Y' || ch == 'Z') term.sign |= uint64_t(1) << b;
                    if (ch == 'Y') ny++;
                    PL_ABORT_IF(ch != 'X' && ch != 'Y' && ch != 'Z' && ch != 'I', "bad Pauli letter");
                }
                cd cc(t.coeff, 0.0);
                for (int q = 0; q < (ny & 3); q++) cc *= cd(0, 1);
                term.cr = cc.real();
                term.ci = cc.imag();
                ht.push_back(term);
            }
            // terms sharing a flip mask are adjacent: the kernel transforms each flip group once
            std::stable_sort(ht.begin() + rec.obs_off, ht.end(),
                             [](const lgpu_bterm_t &x, const lgpu_bterm_t &y) { return x.tflip < y.tflip; });
            rec.obs_cnt = uint32_t(c.obs.size());
            hc.push_back(rec);
            cost[ci] = work;
        }
        std::vector<uint32_t> order(circuits_.size());
        std::iota(order.begin(), order.end(), 0u);
        std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return cost[a] > cost[b]; });
        ngates_ = hg.size();
        nblocks_ = hb.size();
        // device buffers
        int sms = 0;
        PL_LGPU_IS_SUCCESS(lgpu_device_sm_count(0, &sms));
        grid_used_ = unsigned(grid_ > 0 ? grid_ : sms);
        grid_used_ = std::min<unsigned>(grid_used_, unsigned(circuits_.size()));
        const size_t amp = std::is_same_v<Precision, double> ? 16 : 8;
        scratch_amps_ = max_big ? (size_t(1) << max_big) : 0;
        d_circ_ = upload(hc);
        d_order_ = upload(order);
        d_blocks_ = upload(hb);
        d_gates_ = upload(hg);
        d_terms_ = upload(ht.empty() ? std::vector<lgpu_bterm_t>(1) : ht);
        if (pool.empty()) pool.resize(16);
        d_pool_ = upload(pool);
        d_params_ = alloc(std::max<size_t>(params_.size(), 1) * sizeof(double));
        d_out_ = alloc(circuits_.size() * sizeof(double));
        d_counter_ = alloc(256);
        if (scratch_amps_) d_scratch_ = alloc(size_t(grid_used_) * scratch_amps_ * amp);
        PL_LGPU_IS_SUCCESS(lgpu_host_alloc_pinned(&h_params_, std::max<size_t>(params_.size(), 1) * sizeof(double)));
        PL_LGPU_IS_SUCCESS(lgpu_host_alloc_pinned(&h_out_, circuits_.size() * sizeof(double)));
        std::memcpy(h_params_, params_.data(), params_.size() * sizeof(double));
        args_ = lgpu_batch_args_t{};
        args_.circuits = static_cast<const lgpu_bcircuit_t *>(d_circ_);
        args_.order = static_cast<const uint32_t *>(d_order_);
        args_.ncircuits = uint32_t(circuits_.size());
        args_.kmax = uint32_t(kmax_);
        args_.blocks = static_cast<const lgpu_bblock_t *>(d_blocks_);
        args_.gates = static_cast<const lgpu_bgate_t *>(d_gates_);
        args_.pool = static_cast<const double *>(d_pool_);
        args_.terms = static_cast<const lgpu_bterm_t *>(d_terms_);
        args_.scratch = d_scratch_;
        args_.scratch_amps = scratch_amps_;
        args_.counter = static_cast<unsigned *>(d_counter_);
        args_.out = static_cast<double *>(d_out_);
        args_.threads = uint32_t(threads_);
        args_.klarge = uint32_t(klarge());
        if (capture) {
            enqueue();
            PL_LGPU_IS_SUCCESS(lgpu_stream_sync(stream_));
            PL_LGPU_IS_SUCCESS(lgpu_graph_begin(stream_));
            enqueue();
            PL_LGPU_IS_SUCCESS(lgpu_graph_end(stream_, &graph_));
        }
        prepared_ = true;
    }

    // Replay the captured graph; `params` (optional) replaces the parameter vector.
    std::vector<double> run(const std::vector<double> *params = nullptr) {
        launchAsync(params);
        return wait();
    }
    void launchAsync(const std::vector<double> *params = nullptr) {
        PL_ABORT_IF(!prepared_, "run() before prepare()");
        if (params) {
            PL_ABORT_IF(params->size() != params_.size(), "parameter vector has the wrong length");
            std::memcpy(h_params_, params->data(), params->size() * sizeof(double));
        }
        if (graph_)
            PL_LGPU_IS_SUCCESS(lgpu_graph_launch(graph_, stream_));
        else
            enqueue();
    }
    std::vector<double> wait() {
        PL_LGPU_IS_SUCCESS(lgpu_stream_sync(stream_));
        int code = 0;
        PL_LGPU_IS_SUCCESS(lgpu_stream_error(stream_, &code, 1));
        PL_ABORT_IF(code != 0, "A batched kernel timed out waiting for a bulk copy; results are invalid");
        std::vector<double> out(circuits_.size());
        std::memcpy(out.data(), h_out_, out.size() * sizeof(double));
        return out;
    }

    const std::vector<double> &params() const { return params_; }
    size_t numGates() const { return ngates_; }
    size_t numBlocks() const { return nblocks_; }
    unsigned grid() const { return grid_used_; }
    size_t scratchBytes() const {
        return size_t(grid_used_) * scratch_amps_ * (std::is_same_v<Precision, double> ? 16 : 8);
    }

  private:
    struct Op {
        std::vector<int> tgts, ctrls, cvals;
        uint8_t kind = 0, pkind = 0;
        bool adjoint = false;
        int32_t param = -1;              // relative to the circuit's parameter offset
        std::vector<cd> matrix;          // fixed gates (already adjointed)
    };
    using Blocks = std::vector<std::pair<std::vector<int>, std::vector<size_t>>>;
    // A lowered circuit structure: its operations (parameter indices relative
    // to the circuit's first parameter), observable and fused blocks.
    struct Shape {
        size_t n = 0;
        size_t nparams = 0;
        std::vector<Op> ops;
        std::vector<PTerm> obs;
        bool planned = false;
        Blocks blocks;
    };
    struct Circuit {
        std::shared_ptr<Shape> shape;
        size_t param_off = 0;
    };

    // Lower a circuit; its parametric gates' parameters are appended to `pvec`.
    std::shared_ptr<Shape> makeShape(size_t n, const std::vector<std::string> &names,
                                     const std::vector<std::vector<size_t>> &wires,
                                     const std::vector<std::vector<double>> &params, const std::vector<bool> &inverses,
                                     const std::vector<PTerm> &observable, std::vector<double> &pvec) {
        PL_ABORT_IF(n < 1 || n > 30, "batched circuits must have 1..30 qubits");
        PL_ABORT_IF(names.size() != wires.size() || names.size() != params.size() || names.size() != inverses.size(),
                    "names, wires, params and inverses must have the same length");
        auto sh = std::make_shared<Shape>();
        sh->n = n;
        const size_t base = pvec.size();
        sh->ops.reserve(names.size());
        for (size_t i = 0; i < names.size(); i++)
            sh->ops.push_back(lowerOp(n, names[i], wires[i], params[i], inverses[i], pvec, base));
        for (const auto &t : observable) {
            PL_ABORT_IF(t.word.size() != t.wires.size(), "Pauli word and wires differ in length");
            for (size_t w : t.wires) PL_ABORT_IF(w >= n, "observable wire out of range");
            sh->obs.push_back(t);
        }
        sh->nparams = pvec.size() - base;
        return sh;
    }

    // Plan every distinct unplanned shape, on up to 16 host threads (a batch of
    // distinct circuits has as many shapes as circuits; planning one touches
    // only that shape).  An error in any shape is raised here.
    void planShapes() {
        std::vector<Shape *> todo;
        for (const auto &c : circuits_)
            if (!c.shape->planned) todo.push_back(c.shape.get());
        std::sort(todo.begin(), todo.end());
        todo.erase(std::unique(todo.begin(), todo.end()), todo.end());
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const size_t nthreads = std::min<size_t>({size_t(16), size_t(hw), (todo.size() + 63) / 64});
        if (nthreads <= 1) {
            for (Shape *sh : todo) planBlocks(*sh);
            return;
        }
        std::atomic<size_t> next{0};
        std::vector<std::exception_ptr> errs(nthreads);
        std::vector<std::thread> pool;
        for (size_t t = 0; t < nthreads; t++)
            pool.emplace_back([&, t] {
                try {
                    for (size_t i = next.fetch_add(1); i < todo.size(); i = next.fetch_add(1)) planBlocks(*todo[i]);
                } catch (...) {
                    errs[t] = std::current_exception();
                    next.store(todo.size());
                }
            });
        for (auto &th : pool) th.join();
        for (auto &e : errs)
            if (e) std::rethrow_exception(e);
    }

    // Fused blocks of a shape (computed on first use): one block holding the
    // whole state when n <= kmax; otherwise tiles of klarge() bits, with a last
    // block whose tiles cover the observable's flip bits.
    const Blocks &planBlocks(Shape &c) {
        if (c.planned) return c.blocks;
        Blocks &blocks = c.blocks;
        if (int(c.n) <= kmax_) {
            std::vector<int> all(c.n);
            std::iota(all.begin(), all.end(), 0);
            std::vector<size_t> idx(c.ops.size());
            std::iota(idx.begin(), idx.end(), 0);
            blocks.push_back({all, idx});
        } else {
            std::vector<Engine::GateDesc> descs;
            descs.reserve(c.ops.size());
            for (const auto &o : c.ops) {
                Engine::GateDesc d;
                d.kind = Engine::GateDesc::MATRIX;
                d.tgts = o.tgts;
                d.ctrls = o.ctrls;
                descs.push_back(d);
            }
            const auto plan = Engine::plan_fusion(descs, c.n, klarge(), 5, 1);
            for (const auto &b : plan) {
                PL_ABORT_IF(b.tile_bits.empty(), "batched execution: an operation does not fit a fused tile");
                blocks.push_back({b.tile_bits, b.gates});
            }
            // the observable is evaluated on the last block's tiles
            uint64_t flips = 0;
            for (const auto &t : c.obs)
                for (size_t k = 0; k < t.word.size(); k++)
                    if (t.word[k] == 'X' || t.word[k] == 'Y') flips |= uint64_t(1) << Engine::bit_of(c.n, t.wires[k]);
            auto covers = [&](const std::vector<int> &tb) {
                uint64_t m = 0;
                for (int b : tb) m |= uint64_t(1) << b;
                return (flips & ~m) == 0;
            };
            if (blocks.empty() || !covers(blocks.back().first)) {
                std::vector<int> fb;
                for (int b = 0; b < int(c.n); b++)
                    if ((flips >> b) & 1) fb.push_back(b);
                std::vector<int> tile;
                PL_ABORT_IF_NOT(Engine::tile_for(fb, klarge(), 5, c.n, tile),
                                "batched execution: observable flip bits do not fit one tile");
                blocks.push_back({tile, {}});
            }
        }
        c.planned = true;
        return blocks;
    }

    Op lowerOp(size_t n, const std::string &name, const std::vector<size_t> &wires, const std::vector<double> &params,
               bool adjoint, std::vector<double> &pvec, size_t pbase) {
        Engine::GateDesc d = Engine::lower_operation(n, name, wires, adjoint, params, {});
        Op o;
        o.tgts = d.tgts;
        o.ctrls = d.ctrls;
        o.cvals = d.cvals;
        PL_ABORT_IF(d.kind == Engine::GateDesc::IDENTITY, "identity");
        PL_ABORT_IF(d.tgts.size() > 2, ("batched execution supports 1- and 2-target gates, not " + name).c_str());
        PL_ABORT_IF(d.ctrls.size() > 2, "batched execution supports at most 2 controls");
        auto par = [&](uint8_t pk, size_t count) {
            PL_ABORT_IF(params.size() < count, ("missing parameter for " + name).c_str());
            o.pkind = pk;
            o.adjoint = adjoint;
            o.param = int32_t(pvec.size() - pbase);
            for (size_t k = 0; k < count; k++) pvec.push_back(params[k]);
        };
        const std::string base = name;
        if (base == "RX" || base == "CRX") { o.kind = 4; par(1, 1); return o; }
        if (base == "RY" || base == "CRY") { o.kind = 3; par(2, 1); return o; }
        if (base == "RZ" || base == "CRZ") { o.kind = 1; par(3, 1); return o; }
        if (base == "PhaseShift" || base == "ControlledPhaseShift") { o.kind = 1; par(4, 1); return o; }
        if (base == "Rot" || base == "CRot") { o.kind = 0; par(5, 3); return o; }
        if (base == "IsingXX") { o.kind = 5; par(6, 1); return o; }
        if (base == "IsingYY") { o.kind = 5; par(7, 1); return o; }
        if (base == "IsingZZ") { o.kind = 5; par(8, 1); return o; }
        if (d.kind == Engine::GateDesc::PAULI_ROT) {
            std::vector<int> bits;
            std::vector<cd> m;
            PL_ABORT_IF_NOT(Engine::dense_on_bits(d, bits, m, 2), "unsupported Pauli rotation");
            o.matrix = m;
        } else {
            o.matrix = d.matrix;
        }
        if (o.tgts.size() == 1) {
            const auto &m = o.matrix;
            auto z = [](cd v) { return v == cd(0.0); };
            if (m[0] == cd(0.0) && m[3] == cd(0.0) && m[1] == cd(1.0) && m[2] == cd(1.0)) o.kind = 2;
            else if (z(m[1]) && z(m[2])) o.kind = 1;
            else if (m[0].imag() == 0 && m[1].imag() == 0 && m[2].imag() == 0 && m[3].imag() == 0) o.kind = 3;
            else o.kind = 0;
        } else {
            const auto &m = o.matrix;
            bool swap = true;
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 4; c++) {
                    const int target = (r == 0 || r == 3) ? r : 3 - r;
                    if (m[size_t(r * 4 + c)] != cd(c == target ? 1.0 : 0.0)) swap = false;
                }
            o.kind = swap ? 6 : 5;
        }
        return o;
    }

    lgpu_bgate_t record(const Op &o, const std::vector<int> &pos, size_t param_off, std::vector<double> &pool) {
        lgpu_bgate_t g{};
        g.kind = o.kind;
        g.pkind = o.pkind;
        g.q0 = uint8_t(pos[size_t(o.tgts[0])]);
        g.q1 = o.tgts.size() > 1 ? uint8_t(pos[size_t(o.tgts[1])]) : 0;
        PL_ABORT_IF(pos[size_t(o.tgts[0])] < 0 || (o.tgts.size() > 1 && pos[size_t(o.tgts[1])] < 0),
                    "internal: gate target outside its tile");
        for (size_t k = 0; k < o.ctrls.size(); k++) {
            const int b = o.ctrls[k];
            const bool v = o.cvals.empty() ? true : o.cvals[k] != 0;
            if (pos[size_t(b)] >= 0) {
                g.cmask |= 1u << pos[size_t(b)];
                if (v) g.cval |= 1u << pos[size_t(b)];
            } else {
                g.omask |= uint64_t(1) << b;
                if (v) g.oval |= uint64_t(1) << b;
            }
        }
        g.param = o.pkind ? int32_t(param_off) + o.param : -1;
        g.flags = o.adjoint ? 1u : 0u;
        g.mat = uint32_t(pool.size());
        const size_t slot = o.kind >= 5 ? 48 : 16;  // matrix, then the C128 multipliers or the C64 float copy
        pool.resize(pool.size() + slot, 0.0);
        for (size_t e = 0; e < o.matrix.size(); e++) {
            pool[g.mat + 2 * e] = o.matrix[e].real();
            pool[g.mat + 2 * e + 1] = o.matrix[e].imag();
        }
        return g;
    }

    void enqueue() {
        PL_LGPU_IS_SUCCESS(lgpu_memcpy(d_params_, h_params_, std::max<size_t>(params_.size(), 1) * sizeof(double),
                                       LGPU_H2D, 1, stream_));
        PL_LGPU_IS_SUCCESS(lgpu_batch_prepare(static_cast<const lgpu_bgate_t *>(d_gates_), ngates_,
                                              static_cast<const double *>(d_params_), static_cast<double *>(d_pool_),
                                              dt, stream_));
        PL_LGPU_IS_SUCCESS(lgpu_memset(d_counter_, 0, 256, stream_));
        PL_LGPU_IS_SUCCESS(lgpu_batch_run(&args_, dt, grid_used_, stream_));
        PL_LGPU_IS_SUCCESS(lgpu_memcpy(h_out_, d_out_, circuits_.size() * sizeof(double), LGPU_D2H, 1, stream_));
    }

    template <class V> void *upload(const std::vector<V> &v) {
        void *p = alloc(std::max<size_t>(v.size(), 1) * sizeof(V));
        if (!v.empty()) PL_LGPU_IS_SUCCESS(lgpu_memcpy(p, v.data(), v.size() * sizeof(V), LGPU_H2D, 0, stream_));
        return p;
    }
    void *alloc(size_t bytes) {
        void *p = nullptr;
        PL_LGPU_IS_SUCCESS(lgpu_malloc(&p, bytes));
        owned_.push_back(p);
        return p;
    }
    void release() {
        if (graph_) lgpu_graph_destroy(graph_);
        graph_ = nullptr;
        if (stream_) lgpu_stream_sync(stream_);
        for (void *p : owned_) lgpu_free(p);
        owned_.clear();
        if (h_params_) lgpu_host_free_pinned(h_params_);
        if (h_out_) lgpu_host_free_pinned(h_out_);
        h_params_ = h_out_ = nullptr;
    }

    static constexpr size_t kMaxChain = 8;
    int kmax_;
    int threads_;
    int grid_;
    unsigned grid_used_ = 0;
    lgpu_stream_t stream_ = nullptr;
    lgpu_graph_t graph_ = nullptr;
    bool prepared_ = false;
    std::vector<Circuit> circuits_;
    std::vector<std::shared_ptr<Shape>> templates_;
    std::vector<double> params_;
    size_t ngates_ = 0, nblocks_ = 0, scratch_amps_ = 0;
    std::vector<void *> owned_;
    void *d_circ_ = nullptr, *d_order_ = nullptr, *d_blocks_ = nullptr, *d_gates_ = nullptr, *d_terms_ = nullptr,
         *d_pool_ = nullptr, *d_params_ = nullptr, *d_out_ = nullptr, *d_counter_ = nullptr, *d_scratch_ = nullptr;
    void *h_params_ = nullptr, *h_out_ = nullptr;
    lgpu_batch_args_t args_{};
};

} // namespace Pennylane
