// cubff_py.cc — the `cubff` Python module of the GB300 engine, with the
// names of the reference's module (cubff_py.cc:32-96): SimulationParams,
// SimulationState, LanguageInterface, VectorUint8 / VectorUint32 (opaque,
// buffer protocol), GetLanguage, ResetColors and kSelfrepThreshold.
//
//     from cubff_gb300 import cubff
//     lang = cubff.GetLanguage("bff_noheads")
//     lang.RunSimulation(params, None, callback)
#include <pybind11/functional.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>
#include <pybind11/stl_bind.h>

#include <cstdio>

#include "cubff_gb300_sim.h"

namespace py = pybind11;

PYBIND11_MAKE_OPAQUE(std::vector<uint8_t>);
PYBIND11_MAKE_OPAQUE(std::vector<uint32_t>);

PYBIND11_MODULE(cubff, m) {
  m.doc() = "cubff python module (GB300 engine)";

  py::register_exception<cubff::Error>(m, "CubffError");

  py::class_<SimulationParams>(m, "SimulationParams")
      .def(py::init<>())
      .def_readwrite("num_programs", &SimulationParams::num_programs)
      .def_readwrite("seed", &SimulationParams::seed)
      .def_readwrite("mutation_prob", &SimulationParams::mutation_prob)
      .def_readwrite("reset_interval", &SimulationParams::reset_interval)
      .def_readwrite("load_from", &SimulationParams::load_from)
      .def_readwrite("save_to", &SimulationParams::save_to)
      .def_readwrite("callback_interval", &SimulationParams::callback_interval)
      .def_readwrite("save_interval", &SimulationParams::save_interval)
      .def_readwrite("permute_programs", &SimulationParams::permute_programs)
      .def_readwrite("fixed_shuffle", &SimulationParams::fixed_shuffle)
      .def_readwrite("zero_init", &SimulationParams::zero_init)
      .def_readwrite("allowed_interactions", &SimulationParams::allowed_interactions)
      .def_readwrite("eval_selfrep", &SimulationParams::eval_selfrep);

  py::bind_vector<std::vector<uint8_t>>(m, "VectorUint8", py::buffer_protocol());
  py::bind_vector<std::vector<uint32_t>>(m, "VectorUint32", py::buffer_protocol());

  py::class_<SimulationState>(m, "SimulationState")
      .def_readonly("soup", &SimulationState::soup)
      .def_readonly("shuffle_idx", &SimulationState::shuffle_idx)
      .def_readonly("byte_colors", &SimulationState::byte_colors)
      .def_readonly("elapsed_s", &SimulationState::elapsed_s)
      .def_readonly("total_ops", &SimulationState::total_ops)
      .def_readonly("mops_s", &SimulationState::mops_s)
      .def_readonly("epoch", &SimulationState::epoch)
      .def_readonly("ops_per_run", &SimulationState::ops_per_run)
      .def_readonly("brotli_size", &SimulationState::brotli_size)
      .def_readonly("brotli_bpb", &SimulationState::brotli_bpb)
      .def_readonly("bytes_per_prog", &SimulationState::bytes_per_prog)
      .def_readonly("h0", &SimulationState::h0)
      .def_readonly("higher_entropy", &SimulationState::higher_entropy)
      .def_readonly("frequent_bytes", &SimulationState::frequent_bytes)
      .def_readonly("uncommon_bytes", &SimulationState::uncommon_bytes)
      .def_readonly("replication_per_prog", &SimulationState::replication_per_prog);

  py::class_<LanguageInterface>(m, "LanguageInterface")
      .def("PrintProgram",
           [](const LanguageInterface *lang, size_t pc_pos, const std::vector<uint8_t> &program,
              const std::vector<size_t> &separators) {
             lang->PrintProgram(pc_pos, program.data(), program.size(), separators.data(),
                                separators.size());
             fflush(stdout);
           })
      .def("RunSimulation", &LanguageInterface::RunSimulation)
      .def("RunSingleProgram", &LanguageInterface::RunSingleProgram)
      .def("RunSingleParsedProgram", &LanguageInterface::RunSingleParsedProgram)
      .def("EvalSelfrep", &LanguageInterface::EvalSelfrep)
      .def("EvalParsedSelfrep", &LanguageInterface::EvalParsedSelfrep)
      .def("Parse", &LanguageInterface::Parse);

  m.def("GetLanguage", &GetLanguage, py::return_value_policy::reference);
  m.def("ResetColors", []() {
    printf("%s", ResetColors());
    fflush(stdout);
  });
  m.attr("kSelfrepThreshold") = kSelfrepThreshold;
}
