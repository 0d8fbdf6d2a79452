"""Streams Code/RegularMeshBuilder/main.cpp to stdout with the two fixes it
needs to compile and run with g++ (test infrastructure: oracle/build_ref.sh
pipes the result straight into the compiler; nothing is written to disk and
the reference file is not modified):

  * main.cpp:910 binds `auto &found` to the rvalue returned by map::find, an
    MSVC extension; g++ needs `auto found`.
  * WriteMaterials (main.cpp:2144-2163) falls off its end without a return
    value, which is undefined behaviour that g++ -O2 turns into a crash;
    `return 0;` is appended before its closing brace.

usage: ref_fix_rmb.py REFERENCE_ROOT
"""
import sys

path = sys.argv[1] + "/Code/RegularMeshBuilder/main.cpp"
src = open(path, encoding="utf-8", errors="surrogateescape").read()
old = "auto &found = edgesToNumbers.find(edge);"
assert src.count(old) == 1, "unexpected RegularMeshBuilder source"
src = src.replace(old, "auto found = edgesToNumbers.find(edge);")
i = src.index("int WriteMaterials(vector<Material> &materials)")
j = src.index("// Main mesh building and files writing procedure", i)
k = src.rindex("}", i, j)
src = src[:k] + "\treturn 0;\n" + src[k:]
sys.stdout.write(f'#line 1 "{path}"\n')
sys.stdout.write(src)
