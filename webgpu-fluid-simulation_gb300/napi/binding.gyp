{
  "targets": [
    {
      "target_name": "pbf_gb300",
      "sources": ["pbf_addon.cc"],
      "include_dirs": ["../../include"],
      "cflags_cc": ["-std=c++17", "-Wall", "-Wextra"],
      "libraries": [
        "-L<(module_root_dir)/../_build",
        "-lpbf_gb300",
        "-Wl,-rpath,<(module_root_dir)/../_build"
      ]
    }
  ]
}
