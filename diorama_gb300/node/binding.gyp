# Builds diorama.node, the Node-API addon over libdiorama_gb300.so (untested:
# node is not installed on the machines this library was built on). Build the
# library first (python -c "import __graft_entry__ as g; g.build()"), then:
#   node-gyp configure build
{
  "targets": [
    {
      "target_name": "diorama",
      "sources": ["diorama.cc"],
      "include_dirs": ["../../include"],
      "libraries": ["-L<(module_root_dir)/../_build", "-ldiorama_gb300",
                    "-Wl,-rpath,<(module_root_dir)/../_build"],
      "cflags_cc": ["-std=c++17", "-O2"]
    }
  ]
}
