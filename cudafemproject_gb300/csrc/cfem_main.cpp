// cfem_run: command-line driver mirroring the reference's fem/src/main.cpp,
// but taking the run_config path (and optional task names) from argv:
//   cfem_run <run_config.json> [task ...]
// For every task it runs the static or dynamic solve per task_type and writes
// <working_path>/fem_results/<DIM>D/<task>/results.vtk.
#include <cstdio>
#include <iostream>

#include "cfem_femfunc.hpp"

int main(int argc, char **argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s <run_config.json> [task ...]\n", argv[0]);
    return 2;
  }
  try {
    std::vector<std::string> tasks;
    for (int i = 2; i < argc; ++i) tasks.push_back(argv[i]);
    if (tasks.empty()) tasks = cfem_ref::readTaskList(argv[1]);
    if (tasks.empty()) {
      std::fprintf(stderr, "no task given and none listed under \"task\" in %s\n", argv[1]);
      return 2;
    }
    for (const std::string &t : tasks) {
      cfem_ref::dataKeeper dk(argv[1], t);
      dk.ShowInfo();
      if (dk.getTaskType() == "dynamic")
        cfem_ref::gpuCalculateFEM_DYN(cfem_ref::GB300, dk, true);
      else
        cfem_ref::gpuCalculateFEM_EbE_vec(cfem_ref::GB300, dk, true);
      cfem_ref::WriteResults(dk);
      std::cout << "results: " << dk.getDataPaths().output_vtk << "\n";
    }
  } catch (const cfem_ref::Error &e) {
    std::fprintf(stderr, "error (status %d): %s\n", (int)e.status, e.what());
    return 1;
  }
  return 0;
}
