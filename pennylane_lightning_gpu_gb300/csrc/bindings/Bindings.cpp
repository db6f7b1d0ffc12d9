// pybind11 module `lightning_gpu_qubit_ops`: the same classes, method names
// and argument meanings as the reference module
// (src/bindings/Bindings.cpp:67-884, 1727-1788).  Long-running calls release
// the GIL so that several Python threads can drive independent states.
#include <pybind11/complex.h>
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <sstream>

#include "AdjointDiffGPU.hpp"
#include "BatchedExecutor.hpp"

namespace py = pybind11;
using namespace Pennylane;
using namespace Pennylane::Algorithms;
using Pennylane::CUDA::DevTag;
using std::complex;
using std::string;
using std::vector;

namespace {

// Device pool stand-in (reference DevicePool.hpp): one process, one GPU.
class DevPool {
  public:
    DevPool() {
        int n = cuUtil::getGPUCount();
        for (int i = 0; i < n; i++) free_.push_back(i);
    }
    std::vector<int> getActiveDevices() const { return active_; }
    bool isActive(int id) const { return std::find(active_.begin(), active_.end(), id) != active_.end(); }
    bool isInactive(int id) const { return !isActive(id); }
    int acquireDevice() {
        PL_ABORT_IF(free_.empty(), "No free devices");
        int id = free_.front();
        free_.erase(free_.begin());
        active_.push_back(id);
        return id;
    }
    void releaseDevice(int id) {
        active_.erase(std::remove(active_.begin(), active_.end(), id), active_.end());
        free_.push_back(id);
    }
    void syncDevice(int id) {
        PL_LGPU_IS_SUCCESS(lgpu_set_device(id));
        PL_LGPU_IS_SUCCESS(lgpu_stream_sync(nullptr));
    }
    static int getTotalDevices() { return cuUtil::getGPUCount(); }
    static std::vector<int> getDeviceUIDs() {
        std::vector<int> v(static_cast<size_t>(getTotalDevices()));
        std::iota(v.begin(), v.end(), 0);
        return v;
    }
    static void setDeviceIdx(int id) { PL_LGPU_IS_SUCCESS(lgpu_set_device(id)); }

  private:
    std::vector<int> free_, active_;
};

template <class PrecisionT, class ParamT> void sv_class_bindings(py::module_ &m) {
    using SV = StateVectorCudaManaged<PrecisionT>;
    using np_arr_r = py::array_t<ParamT, py::array::c_style | py::array::forcecast>;
    using np_arr_c = py::array_t<std::complex<ParamT>, py::array::c_style | py::array::forcecast>;
    using index_type = typename std::conditional<std::is_same<ParamT, float>::value, int32_t, int64_t>::type;
    using np_arr_sparse_ind = py::array_t<index_type, py::array::c_style | py::array::forcecast>;
    const std::string bitsize = std::to_string(sizeof(std::complex<PrecisionT>) * 8);
    std::string class_name = "LightningGPU_C" + bitsize;
    using rel = py::call_guard<py::gil_scoped_release>;

    auto to_cvec = [](const np_arr_c &a) {
        const auto b = a.request();
        std::vector<std::complex<PrecisionT>> v;
        if (b.size) {
            const auto *p = static_cast<const std::complex<PrecisionT> *>(b.ptr);
            v.assign(p, p + b.size);
        }
        return v;
    };

    py::class_<SV> cls(m, class_name.c_str());
    cls.def(py::init<std::size_t>())
        .def(py::init<std::size_t, DevTag<int>>())
        .def(py::init<const SV &>())
        .def(py::init([](const np_arr_c &arr) {
            py::buffer_info info = arr.request();
            return new SV(static_cast<const std::complex<PrecisionT> *>(info.ptr), static_cast<std::size_t>(arr.size()));
        }))
        .def(
            "setBasisState",
            [](SV &sv, const size_t index, const bool use_async) {
                sv.setBasisState(std::complex<PrecisionT>(1, 0), index, use_async);
            },
            "Create Basis State on GPU.")
        .def(
            "setStateVector",
            [](SV &sv, const np_arr_sparse_ind &indices, const np_arr_c &state, const bool use_async) {
                PL_ABORT_IF(indices.size() != state.size(), "indices and values must have the same length");
                sv.template setStateVector<index_type>(static_cast<index_type>(indices.request().size),
                                                       static_cast<std::complex<PrecisionT> *>(state.request().ptr),
                                                       static_cast<index_type *>(indices.request().ptr), use_async);
            },
            "Set State Vector on GPU with values and their corresponding indices for the state vector on device");

    // Per-gate methods: (wires, adjoint, params)
    auto gate0 = [&cls](const char *name, void (SV::*f)(const std::vector<size_t> &, bool)) {
        cls.def(
            name,
            [f](SV &sv, const std::vector<std::size_t> &wires, bool adjoint,
                [[maybe_unused]] const std::vector<ParamT> &params) { (sv.*f)(wires, adjoint); },
            (std::string("Apply the ") + name + " gate.").c_str(), py::call_guard<py::gil_scoped_release>());
    };
    gate0("Identity", &SV::applyIdentity);
    gate0("PauliX", &SV::applyPauliX);
    gate0("PauliY", &SV::applyPauliY);
    gate0("PauliZ", &SV::applyPauliZ);
    gate0("Hadamard", &SV::applyHadamard);
    gate0("S", &SV::applyS);
    gate0("T", &SV::applyT);
    gate0("CNOT", &SV::applyCNOT);
    gate0("SWAP", &SV::applySWAP);
    gate0("CSWAP", &SV::applyCSWAP);
    gate0("Toffoli", &SV::applyToffoli);
    gate0("CY", &SV::applyCY);
    gate0("CZ", &SV::applyCZ);
    auto gate1 = [&cls](const char *name, void (SV::*f)(const std::vector<size_t> &, bool, PrecisionT)) {
        cls.def(
            name,
            [f, name](SV &sv, const std::vector<std::size_t> &wires, bool adjoint, const std::vector<ParamT> &params) {
                PL_ABORT_IF(params.empty(), (std::string(name) + " needs one parameter").c_str());
                (sv.*f)(wires, adjoint, params.front());
            },
            (std::string("Apply the ") + name + " gate.").c_str(), py::call_guard<py::gil_scoped_release>());
    };
    gate1("RX", &SV::applyRX);
    gate1("RY", &SV::applyRY);
    gate1("RZ", &SV::applyRZ);
    gate1("PhaseShift", &SV::applyPhaseShift);
    gate1("ControlledPhaseShift", &SV::applyControlledPhaseShift);
    gate1("CRX", &SV::applyCRX);
    gate1("CRY", &SV::applyCRY);
    gate1("CRZ", &SV::applyCRZ);
    gate1("IsingXX", &SV::applyIsingXX);
    gate1("IsingYY", &SV::applyIsingYY);
    gate1("IsingZZ", &SV::applyIsingZZ);
    gate1("MultiRZ", &SV::applyMultiRZ);
    gate1("SingleExcitation", &SV::applySingleExcitation);
    gate1("SingleExcitationMinus", &SV::applySingleExcitationMinus);
    gate1("SingleExcitationPlus", &SV::applySingleExcitationPlus);
    gate1("DoubleExcitation", &SV::applyDoubleExcitation);
    gate1("DoubleExcitationMinus", &SV::applyDoubleExcitationMinus);
    gate1("DoubleExcitationPlus", &SV::applyDoubleExcitationPlus);
    cls.def(
        "Rot",
        [](SV &sv, const std::vector<std::size_t> &wires, bool adjoint, const std::vector<ParamT> &params) {
            PL_ABORT_IF(params.size() != 3, "Rot needs three parameters");
            sv.applyRot(wires, adjoint, params);
        },
        "Apply the Rot gate.", rel());
    cls.def(
        "CRot",
        [](SV &sv, const std::vector<std::size_t> &wires, bool adjoint, const std::vector<ParamT> &params) {
            PL_ABORT_IF(params.size() != 3, "CRot needs three parameters");
            sv.applyCRot(wires, adjoint, params);
        },
        "Apply the CRot gate.", rel());

    cls.def("apply",
            py::overload_cast<const vector<string> &, const vector<vector<std::size_t>> &, const vector<bool> &,
                              const vector<vector<PrecisionT>> &>(&SV::applyOperation),
            rel())
        .def("apply",
             py::overload_cast<const vector<string> &, const vector<vector<std::size_t>> &, const vector<bool> &>(
                 &SV::applyOperation),
             rel())
        .def("apply",
             py::overload_cast<const std::string &, const vector<size_t> &, bool, const vector<PrecisionT> &,
                               const std::vector<std::complex<PrecisionT>> &>(&SV::applyOperation_std),
             rel());

    cls.def(
           "ExpectationValue",
           [to_cvec](SV &sv, const std::string &obsName, const std::vector<std::size_t> &wires,
                     [[maybe_unused]] const std::vector<ParamT> &params, const np_arr_c &gate_matrix) {
               auto m = to_cvec(gate_matrix);
               py::gil_scoped_release r;
               return sv.expval(obsName, wires, params, m).x;
           },
           "Calculate the expectation value of the given observable.")
        .def(
            "ExpectationValue",
            [to_cvec](SV &sv, const std::vector<std::string> &obsName, const std::vector<std::size_t> &wires,
                      [[maybe_unused]] const std::vector<std::vector<ParamT>> &params, const np_arr_c &gate_matrix) {
                std::string obs_concat{"#"};
                for (const auto &sub : obsName) obs_concat += sub;
                auto m = to_cvec(gate_matrix);
                py::gil_scoped_release r;
                return sv.expval(obs_concat, wires, std::vector<PrecisionT>{}, m).x;
            },
            "Calculate the expectation value of the given observable.")
        .def(
            "ExpectationValue",
            [to_cvec](SV &sv, const std::vector<std::size_t> &wires, const np_arr_c &gate_matrix) {
                auto m = to_cvec(gate_matrix);
                py::gil_scoped_release r;
                return sv.expval(wires, m).x;
            },
            "Calculate the expectation value of a Hamiltonian given as a dense matrix.")
        .def(
            "ExpectationValue",
            [](SV &sv, const np_arr_sparse_ind &csrOffsets, const np_arr_sparse_ind &columns, const np_arr_c values) {
                return sv.template getExpectationValueOnSparseSpMV<index_type>(
                    static_cast<index_type *>(csrOffsets.request().ptr), static_cast<index_type>(csrOffsets.request().size),
                    static_cast<index_type *>(columns.request().ptr),
                    static_cast<std::complex<PrecisionT> *>(values.request().ptr),
                    static_cast<index_type>(values.request().size));
            },
            "Calculate the expectation value of a sparse Hamiltonian.")
        .def(
            "ExpectationValue",
            [](SV &sv, const std::vector<std::string> &pauli_words, const std::vector<std::vector<std::size_t>> &target_wires,
               const np_arr_c &coeffs) {
                PL_ABORT_IF(size_t(coeffs.size()) != pauli_words.size(), "Number of coefficients and words differ");
                auto *data_ptr = static_cast<const complex<PrecisionT> *>(coeffs.request().ptr);
                std::vector<complex<PrecisionT>> c(data_ptr, data_ptr + coeffs.size());
                py::gil_scoped_release r;
                return sv.getExpectationValuePauliWords(pauli_words, target_wires, c.data());
            },
            "Calculate the expectation value of a Hamiltonian composed solely from sums of Pauli-words")
        .def(
            "Probability",
            [](SV &sv, const std::vector<std::size_t> &wires) {
                std::vector<double> p;
                {
                    py::gil_scoped_release r;
                    p = sv.probability(wires);
                }
                py::array_t<ParamT> out(p.size());
                auto *o = out.mutable_data();
                for (size_t i = 0; i < p.size(); i++) o[i] = static_cast<ParamT>(p[i]);
                return out;
            },
            "Calculate the probabilities for given wires. Results returned in Col-major order.")
        .def("GenerateSamples",
             [](SV &sv, size_t num_wires, size_t num_shots) {
                 std::vector<size_t> result;
                 {
                     py::gil_scoped_release r;
                     result = sv.generate_samples(num_shots);
                 }
                 PL_ABORT_IF(num_wires != sv.getNumQubits(), "num_wires must equal the number of qubits");
                 py::array_t<size_t> out({num_shots, num_wires});
                 std::copy(result.begin(), result.end(), out.mutable_data());
                 return out;
             })
        .def(
            "DeviceToDevice", [](SV &sv, const SV &other, bool async) { sv.updateData(other, async); },
            "Synchronize data from another GPU device to current device.")
        .def(
            "DeviceToHost",
            [](const SV &gpu_sv, np_arr_c &cpu_sv, bool) {
                py::buffer_info info = cpu_sv.request();
                auto *data_ptr = static_cast<complex<PrecisionT> *>(info.ptr);
                if (cpu_sv.size()) gpu_sv.CopyGpuDataToHost(data_ptr, size_t(cpu_sv.size()));
            },
            "Synchronize data from the GPU device to host.")
        .def(
            "HostToDevice",
            [](SV &gpu_sv, const np_arr_c &cpu_sv, bool async) {
                const py::buffer_info info = cpu_sv.request();
                const auto *data_ptr = static_cast<complex<PrecisionT> *>(info.ptr);
                const auto length = static_cast<size_t>(info.size);
                if (length) gpu_sv.CopyHostDataToGpu(data_ptr, length, async);
            },
            "Synchronize data from the host device to GPU.")
        .def("GetNumGPUs", &cuUtil::getGPUCount, "Get the number of available GPUs.")
        .def("getCurrentGPU", &cuUtil::getGPUIdx, "Get the GPU index for the statevector data.")
        .def("numQubits", &SV::getNumQubits)
        .def("dataLength", &SV::getLength)
        .def("resetGPU", [](SV &sv) { sv.initSV(); });

    // ---- extensions of this engine (not in the reference module) ----------
    cls.def("setSeed", &SV::setSeed, "Fix the seed of the sampler's std::mt19937 stream.")
        .def("clearSeed", &SV::clearSeed)
        .def("setFusion", &SV::setFusion, py::arg("on"), py::arg("tile_bits") = 0, py::arg("min_low_bits") = 0,
             "Enable/disable shared-memory gate fusion for multi-op apply(); optionally set the tile size and "
             "the shortest contiguous low run of a tile (in bits).")
        .def("getFusion", &SV::getFusion)
        .def(
            "GenerateSampleIndices",
            [](SV &sv, size_t num_shots, bool sorted) {
                std::vector<uint64_t> idx;
                {
                    py::gil_scoped_release r;
                    idx = sv.generate_sample_indices(num_shots, sorted);
                }
                py::array_t<uint64_t> out(idx.size());
                std::copy(idx.begin(), idx.end(), out.mutable_data());
                return out;
            },
            py::arg("num_shots"), py::arg("sorted") = true, "Sampled basis-state indices.")
        .def(
            "GetState",
            [](const SV &sv) {
                py::array_t<std::complex<PrecisionT>> out(sv.getLength());
                {
                    py::gil_scoped_release r;
                    sv.CopyGpuDataToHost(out.mutable_data(), sv.getLength());
                }
                return out;
            },
            "Copy the state to a new numpy array.")
        .def(
            "PauliWordExpectations",
            [](SV &sv, const std::vector<std::string> &words, const std::vector<std::vector<size_t>> &wires) {
                std::vector<uint64_t> flip, sgn;
                std::vector<uint8_t> ny;
                sv.pauliMasks(words, wires, flip, sgn, ny);
                std::vector<double> ev(words.size());
                if (!ev.empty()) {
                    py::gil_scoped_release r;
                    PL_LGPU_IS_SUCCESS(lgpu_expval_pauli_words(sv.ctx(), sv.getData(), sv.nq(), SV::dt(),
                                                               uint32_t(ev.size()), flip.data(), sgn.data(), ny.data(),
                                                               ev.data(), 0, sv.lstream()));
                }
                return ev;
            },
            "Per-word <P_j> in FP64.")
        .def(
            "ApplyGeneratorOf",
            [](SV &sv, const std::string &name, const std::vector<size_t> &wires, bool adj) {
                return sv.applyGeneratorOf(name, wires, adj);
            },
            "Apply the generator of a parametric gate; returns its scale factor.")
        .def("synchronize", &SV::sync, rel())
        .def(
            "dataPtr", [](SV &sv) { return reinterpret_cast<uintptr_t>(sv.getData()); },
            "Device address of the amplitudes.")
        .def(
            "streamPtr", [](SV &sv) { return reinterpret_cast<uintptr_t>(sv.getStream()); },
            "The CUDA stream the state works on.")
        .def(
            "copyFrom",
            [](SV &sv, const SV &other) {
                PL_ABORT_IF(other.getNumQubits() != sv.getNumQubits(), "States of different sizes");
                py::gil_scoped_release r;
                sv.updateData(other, false);
            },
            "Copy the amplitudes of another state of the same size (device to device).");

    // ---- observables -------------------------------------------------------
    class_name = "ObservableGPU_C" + bitsize;
    py::class_<ObservableGPU<PrecisionT>, std::shared_ptr<ObservableGPU<PrecisionT>>>(m, class_name.c_str(),
                                                                                      py::module_local())
        .def(
            "applyInPlace",
            [](const ObservableGPU<PrecisionT> &obs, SV &sv) {
                py::gil_scoped_release r;
                obs.applyInPlace(sv);
                sv.sync();
            },
            "O|psi> in place (ObservableGPU::applyInPlace; not bound by the reference module).");

    class_name = "NamedObsGPU_C" + bitsize;
    py::class_<NamedObsGPU<PrecisionT>, std::shared_ptr<NamedObsGPU<PrecisionT>>, ObservableGPU<PrecisionT>>(
        m, class_name.c_str(), py::module_local())
        .def(py::init([](const std::string &name, const std::vector<size_t> &wires) {
            return NamedObsGPU<PrecisionT>(name, wires);
        }))
        .def("__repr__", &NamedObsGPU<PrecisionT>::getObsName)
        .def("get_wires", &NamedObsGPU<PrecisionT>::getWires, "Get wires of observables")
        .def(
            "__eq__",
            [](const NamedObsGPU<PrecisionT> &self, py::handle other) -> bool {
                if (!py::isinstance<NamedObsGPU<PrecisionT>>(other)) return false;
                auto other_cast = other.cast<NamedObsGPU<PrecisionT>>();
                return self == other_cast;
            },
            "Compare two observables");

    class_name = "HermitianObsGPU_C" + bitsize;
    py::class_<HermitianObsGPU<PrecisionT>, std::shared_ptr<HermitianObsGPU<PrecisionT>>, ObservableGPU<PrecisionT>>(
        m, class_name.c_str(), py::module_local())
        .def(py::init([to_cvec](const np_arr_c &matrix, const std::vector<size_t> &wires) {
            return HermitianObsGPU<PrecisionT>(to_cvec(matrix), wires);
        }))
        .def("__repr__", &HermitianObsGPU<PrecisionT>::getObsName)
        .def("get_wires", &HermitianObsGPU<PrecisionT>::getWires, "Get wires of observables")
        .def(
            "__eq__",
            [](const HermitianObsGPU<PrecisionT> &self, py::handle other) -> bool {
                if (!py::isinstance<HermitianObsGPU<PrecisionT>>(other)) return false;
                auto other_cast = other.cast<HermitianObsGPU<PrecisionT>>();
                return self == other_cast;
            },
            "Compare two observables");

    class_name = "TensorProdObsGPU_C" + bitsize;
    py::class_<TensorProdObsGPU<PrecisionT>, std::shared_ptr<TensorProdObsGPU<PrecisionT>>, ObservableGPU<PrecisionT>>(
        m, class_name.c_str(), py::module_local())
        .def(py::init([](const std::vector<std::shared_ptr<ObservableGPU<PrecisionT>>> &obs) {
            return TensorProdObsGPU<PrecisionT>(obs);
        }))
        .def("__repr__", &TensorProdObsGPU<PrecisionT>::getObsName)
        .def("get_wires", &TensorProdObsGPU<PrecisionT>::getWires, "Get wires of observables")
        .def(
            "__eq__",
            [](const TensorProdObsGPU<PrecisionT> &self, py::handle other) -> bool {
                if (!py::isinstance<TensorProdObsGPU<PrecisionT>>(other)) return false;
                auto other_cast = other.cast<TensorProdObsGPU<PrecisionT>>();
                return self == other_cast;
            },
            "Compare two observables");

    class_name = "HamiltonianGPU_C" + bitsize;
    using ObsPtr = std::shared_ptr<ObservableGPU<PrecisionT>>;
    py::class_<HamiltonianGPU<PrecisionT>, std::shared_ptr<HamiltonianGPU<PrecisionT>>, ObservableGPU<PrecisionT>>(
        m, class_name.c_str(), py::module_local())
        .def(py::init([](const np_arr_r &coeffs, const std::vector<ObsPtr> &obs) {
            auto buffer = coeffs.request();
            const auto ptr = static_cast<const ParamT *>(buffer.ptr);
            PL_ABORT_IF(size_t(buffer.size) != obs.size(), "Number of coefficients and observables differ");
            return HamiltonianGPU<PrecisionT>{std::vector<PrecisionT>(ptr, ptr + buffer.size), obs};
        }))
        .def("__repr__", &HamiltonianGPU<PrecisionT>::getObsName)
        .def("get_wires", &HamiltonianGPU<PrecisionT>::getWires, "Get wires of observables")
        .def(
            "__eq__",
            [](const HamiltonianGPU<PrecisionT> &self, py::handle other) -> bool {
                if (!py::isinstance<HamiltonianGPU<PrecisionT>>(other)) return false;
                auto other_cast = other.cast<HamiltonianGPU<PrecisionT>>();
                return self == other_cast;
            },
            "Compare two observables");

    class_name = "SparseHamiltonianGPU_C" + bitsize;
    using SpIDX = typename SparseHamiltonianGPU<PrecisionT>::IdxT;
    py::class_<SparseHamiltonianGPU<PrecisionT>, std::shared_ptr<SparseHamiltonianGPU<PrecisionT>>,
               ObservableGPU<PrecisionT>>(m, class_name.c_str(), py::module_local())
        .def(py::init([](const np_arr_c &data, const np_arr_sparse_ind &indices, const np_arr_sparse_ind &offsets,
                         const std::vector<std::size_t> &wires) {
            const auto *data_ptr = static_cast<const complex<PrecisionT> *>(data.request().ptr);
            const auto *indices_ptr = static_cast<const SpIDX *>(indices.request().ptr);
            const auto *offsets_ptr = static_cast<const SpIDX *>(offsets.request().ptr);
            return SparseHamiltonianGPU<PrecisionT>{
                std::vector<complex<PrecisionT>>(data_ptr, data_ptr + data.size()),
                std::vector<SpIDX>(indices_ptr, indices_ptr + indices.size()),
                std::vector<SpIDX>(offsets_ptr, offsets_ptr + offsets.size()), wires};
        }))
        .def("__repr__", &SparseHamiltonianGPU<PrecisionT>::getObsName)
        .def("get_wires", &SparseHamiltonianGPU<PrecisionT>::getWires, "Get wires of observables")
        .def(
            "__eq__",
            [](const SparseHamiltonianGPU<PrecisionT> &self, py::handle other) -> bool {
                if (!py::isinstance<SparseHamiltonianGPU<PrecisionT>>(other)) return false;
                auto other_cast = other.cast<SparseHamiltonianGPU<PrecisionT>>();
                return self == other_cast;
            },
            "Compare two observables");

    // ---- ops + adjoint -----------------------------------------------------
    class_name = "OpsStructGPU_C" + bitsize;
    py::class_<OpsData<SV>>(m, class_name.c_str(), py::module_local())
        .def(py::init<const std::vector<std::string> &, const std::vector<std::vector<ParamT>> &,
                      const std::vector<std::vector<size_t>> &, const std::vector<bool> &,
                      const std::vector<std::vector<std::complex<PrecisionT>>> &>())
        .def("__repr__", [](const OpsData<SV> &ops) {
            std::ostringstream s;
            for (size_t op = 0; op < ops.getSize(); op++) {
                s << "{'name': " << ops.getOpsName()[op] << ", 'params': ";
                print_vec(s, ops.getOpsParams()[op]);
                s << ", 'inv': " << ops.getOpsInverses()[op] << "}";
                if (op < ops.getSize() - 1) s << ",";
            }
            return "Operations: [" + s.str() + "]";
        });

    class_name = "AdjointJacobianGPU_C" + bitsize;
    py::class_<AdjointJacobianGPU<PrecisionT>>(m, class_name.c_str(), py::module_local())
        .def(py::init<>())
        .def("create_ops_list",
             [](AdjointJacobianGPU<PrecisionT> &adj, const std::vector<std::string> &ops_name,
                const std::vector<np_arr_r> &ops_params, const std::vector<std::vector<size_t>> &ops_wires,
                const std::vector<bool> &ops_inverses, const std::vector<np_arr_c> &ops_matrices) {
                 static_cast<void>(adj);
                 std::vector<std::vector<PrecisionT>> conv_params(ops_params.size());
                 std::vector<std::vector<std::complex<PrecisionT>>> conv_matrices(ops_matrices.size());
                 for (size_t op = 0; op < ops_name.size(); op++) {
                     const auto p_buffer = ops_params[op].request();
                     const auto m_buffer = ops_matrices[op].request();
                     if (p_buffer.size) {
                         const auto *p_ptr = static_cast<const ParamT *>(p_buffer.ptr);
                         conv_params[op] = std::vector<PrecisionT>{p_ptr, p_ptr + p_buffer.size};
                     }
                     if (m_buffer.size) {
                         const auto *m_ptr = static_cast<const std::complex<ParamT> *>(m_buffer.ptr);
                         conv_matrices[op] = std::vector<std::complex<PrecisionT>>{m_ptr, m_ptr + m_buffer.size};
                     }
                 }
                 return OpsData<SV>{ops_name, conv_params, ops_wires, ops_inverses, conv_matrices};
             })
        .def(
            "adjoint_jacobian",
            [](AdjointJacobianGPU<PrecisionT> &adj, const SV &sv,
               const std::vector<std::shared_ptr<ObservableGPU<PrecisionT>>> &observables, const OpsData<SV> &operations,
               const std::vector<size_t> &trainableParams) {
                std::vector<std::vector<PrecisionT>> jac(observables.size(),
                                                         std::vector<PrecisionT>(trainableParams.size(), 0));
                {
                    py::gil_scoped_release r;
                    adj.adjointJacobian(sv.getData(), sv.getLength(), jac, observables, operations, trainableParams,
                                        false, sv.getDataBuffer().getDevTag());
                }
                return py::array_t<ParamT>(py::cast(jac));
            })
        .def(
            "adjoint_jacobian_batched",
            [](AdjointJacobianGPU<PrecisionT> &adj, const SV &sv,
               const std::vector<std::shared_ptr<ObservableGPU<PrecisionT>>> &observables, const OpsData<SV> &operations,
               const std::vector<size_t> &trainableParams) {
                std::vector<std::vector<PrecisionT>> jac(observables.size(),
                                                         std::vector<PrecisionT>(trainableParams.size(), 0));
                {
                    py::gil_scoped_release r;
                    adj.batchAdjointJacobian(sv.getData(), sv.getLength(), jac, observables, operations,
                                             trainableParams, false);
                }
                return py::array_t<ParamT>(py::cast(jac));
            });
}

// Operations as the Python list of (name, wires, params[, inverse]) tuples and
// the observable as (coeff, word, wires) terms, unpacked in one pass here
// (wires and params: any iterables of integers and numbers).
struct BatchOps {
    std::vector<std::string> names;
    std::vector<std::vector<size_t>> wires;
    std::vector<std::vector<double>> params;
    std::vector<bool> inverses;
};

inline BatchOps unpack_batch_ops(const py::sequence &ops) {
    BatchOps L;
    const size_t n = py::len(ops);
    L.names.reserve(n);
    L.wires.reserve(n);
    L.params.reserve(n);
    L.inverses.reserve(n);
    for (py::handle h : ops) {
        const auto o = py::reinterpret_borrow<py::sequence>(h);
        const size_t len = py::len(o);
        PL_ABORT_IF(len < 3, "an operation is (name, wires, params[, inverse])");
        L.names.push_back(o[0].cast<std::string>());
        std::vector<size_t> w;
        for (py::handle x : py::object(o[1])) w.push_back(x.cast<size_t>());
        std::vector<double> p;
        for (py::handle x : py::object(o[2])) p.push_back(x.cast<double>());
        L.wires.push_back(std::move(w));
        L.params.push_back(std::move(p));
        L.inverses.push_back(len > 3 ? py::object(o[3]).cast<bool>() : false);
    }
    return L;
}

template <class Term> std::vector<Term> unpack_batch_terms(const py::sequence &obs) {
    std::vector<Term> terms;
    terms.reserve(py::len(obs));
    for (py::handle h : obs) {
        const auto t = py::reinterpret_borrow<py::sequence>(h);
        PL_ABORT_IF(py::len(t) != 3, "an observable term is (coeff, word, wires)");
        std::vector<size_t> w;
        for (py::handle x : py::object(t[2])) w.push_back(x.cast<size_t>());
        terms.push_back({py::object(t[0]).cast<double>(), py::object(t[1]).cast<std::string>(), std::move(w)});
    }
    return terms;
}

template <class PrecisionT> void batched_bindings(py::module_ &m) {
    using BE = BatchedExecutor<PrecisionT>;
    const std::string name = std::string("BatchedExecutor_C") + (std::is_same_v<PrecisionT, double> ? "128" : "64");
    py::class_<BE>(m, name.c_str())
        .def(py::init<int, int, int>(), py::arg("kmax") = 0, py::arg("threads") = 256, py::arg("grid") = 0)
        .def(
            "add_circuit",
            [](BE &be, size_t n, const py::sequence &ops, const py::sequence &obs) {
                const BatchOps L = unpack_batch_ops(ops);
                const auto terms = unpack_batch_terms<typename BE::PTerm>(obs);
                return be.addCircuit(n, L.names, L.wires, L.params, L.inverses, terms);
            },
            "Add a circuit: ops as (name, wires, params[, inverse]) tuples, observable as (coeff, word, wires) terms.")
        .def(
            "add_template",
            [](BE &be, size_t n, const py::sequence &ops, const py::sequence &obs) {
                const BatchOps L = unpack_batch_ops(ops);
                const auto terms = unpack_batch_terms<typename BE::PTerm>(obs);
                return be.addTemplate(n, L.names, L.wires, L.params, L.inverses, terms);
            },
            "Add a circuit structure shared by many parameter sets (same arguments as add_circuit); returns its id.")
        .def("template_num_params", &BE::templateNumParams)
        .def(
            "add_instances",
            [](BE &be, size_t tid, const py::array_t<double, py::array::c_style | py::array::forcecast> &params) {
                const size_t P = be.templateNumParams(tid);
                PL_ABORT_IF(params.ndim() != 2 || size_t(params.shape(1)) != P,
                            "instance parameters must have shape (count, template_num_params)");
                return be.addInstances(tid, params.data(), size_t(params.shape(0)));
            },
            "Add one circuit per row of `params` (shape (count, template_num_params)); returns the first index.")
        .def("prepare", &BE::prepare, py::arg("capture") = true, py::call_guard<py::gil_scoped_release>(),
             "Plan and upload; with capture=True also run once and capture the CUDA graph that run() replays.")
        .def(
            "run",
            [](BE &be, py::object params) {
                std::vector<double> out;
                if (params.is_none()) {
                    py::gil_scoped_release r;
                    out = be.run(nullptr);
                } else {
                    auto p = params.cast<std::vector<double>>();
                    py::gil_scoped_release r;
                    out = be.run(&p);
                }
                return py::array_t<double>(out.size(), out.data());
            },
            py::arg("params") = py::none(), "Replay the graph and return one result per circuit.")
        .def(
            "launch_async",
            [](BE &be, py::object params) {
                if (params.is_none()) {
                    be.launchAsync(nullptr);
                } else {
                    auto p = params.cast<std::vector<double>>();
                    be.launchAsync(&p);
                }
            },
            py::arg("params") = py::none())
        .def(
            "wait",
            [](BE &be) {
                std::vector<double> out;
                {
                    py::gil_scoped_release r;
                    out = be.wait();
                }
                return py::array_t<double>(out.size(), out.data());
            })
        .def("num_params", &BE::numParams)
        .def("num_circuits", &BE::numCircuits)
        .def("param_offset", &BE::paramOffset)
        .def("params", [](const BE &be) { return be.params(); })
        .def("num_gates", &BE::numGates)
        .def("num_blocks", &BE::numBlocks)
        .def("grid", &BE::grid)
        .def("kmax", &BE::kmax)
        .def("scratch_bytes", &BE::scratchBytes);
}

} // namespace

PYBIND11_MODULE(lightning_gpu_qubit_ops, m) {
    py::options options;
    options.disable_function_signatures();
    py::register_exception<LightningException>(m, "PLException");

    m.def("device_reset", &cuUtil::deviceReset, "Reset all GPU devices and contexts.");
    m.def("allToAllAccess", []() { PL_LGPU_IS_SUCCESS(lgpu_peer_access_all()); });
    m.def("is_gpu_supported", &cuUtil::isCuQuantumSupported, py::arg("device_number") = 0,
          "Checks if the given GPU device is the architecture this engine is built for (sm_103).");
    m.def("get_gpu_arch", &cuUtil::getGPUArch, py::arg("device_number") = 0,
          "Returns the given GPU major and minor GPU support.");
    m.def("abi_version", &lgpu_abi_version);
    m.def(
        "set_f64_mode", [](int mode) { PL_LGPU_IS_SUCCESS(lgpu_set_f64_mode(mode)); },
        "complex128 arithmetic of the streaming gate kernels: 0 native FP64, 1 FP64 FMA + integer-pipe multiplies");
    m.def("get_f64_mode", &lgpu_get_f64_mode);
    m.def(
        "set_stream_mode", [](int mode) { PL_LGPU_IS_SUCCESS(lgpu_set_stream_mode(mode)); },
        "1-target gate kernels: 1 bulk-copy pipelined tiles, 0 grid-stride");
    m.def("get_stream_mode", &lgpu_get_stream_mode);
    m.def(
        "set_tensor_mode", [](int mode) { PL_LGPU_IS_SUCCESS(lgpu_set_tensor_mode(mode)); },
        "1: dense 6-target complex64 gates on the lowest six bits on the tensor cores; 0: FP32 shared-memory kernel.");
    m.def("get_tensor_mode", &lgpu_get_tensor_mode);

    py::class_<DevPool>(m, "DevPool")
        .def(py::init<>())
        .def("getActiveDevices", &DevPool::getActiveDevices)
        .def("isActive", &DevPool::isActive)
        .def("isInactive", &DevPool::isInactive)
        .def("acquireDevice", &DevPool::acquireDevice)
        .def("releaseDevice", &DevPool::releaseDevice)
        .def("syncDevice", &DevPool::syncDevice)
        .def_static("getTotalDevices", &DevPool::getTotalDevices)
        .def_static("getDeviceUIDs", &DevPool::getDeviceUIDs)
        .def_static("setDeviceID", &DevPool::setDeviceIdx);

    py::class_<DevTag<int>>(m, "DevTag")
        .def(py::init<>())
        .def(py::init<int>())
        .def(py::init([](int device_id, void *stream_id) {
            return new DevTag<int>(device_id, static_cast<cudaStream_t>(stream_id));
        }))
        .def(py::init([](int device_id, uintptr_t stream_ptr) {
            // stream given as an integer handle (e.g. torch.cuda.Stream().cuda_stream)
            return new DevTag<int>(device_id, reinterpret_cast<cudaStream_t>(stream_ptr));
        }))
        .def(py::init<const DevTag<int> &>())
        .def("getDeviceID", &DevTag<int>::getDeviceID)
        .def("getStreamID", [](DevTag<int> &dev_tag) { return static_cast<void *>(dev_tag.getStreamID()); })
        .def("refresh", &DevTag<int>::refresh);

    sv_class_bindings<float, float>(m);
    sv_class_bindings<double, double>(m);
    batched_bindings<float>(m);
    batched_bindings<double>(m);
}
