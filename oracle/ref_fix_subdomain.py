"""Streams Code/OutputNu/Subdomain.cpp to stdout with the one fix it needs to
compile with g++ (test infrastructure: oracle/build_ref.sh pipes the result
straight into the compiler; nothing is written to disk and the reference
file is not modified):

  * the `double_eps * double` and `double_eps * double_eps` operators
    (Subdomain.cpp:84-94) take their operands by non-const reference, and
    BuildSigmaStruct multiplies the temporaries that `double_eps -
    double_eps` returns (:760-797): binding a temporary to a non-const
    reference is an MSVC extension; g++ needs const references.  The
    operators only read their operands.

usage: ref_fix_subdomain.py REFERENCE_ROOT
"""
import sys

path = sys.argv[1] + "/Code/OutputNu/Subdomain.cpp"
src = open(path, encoding="utf-8", errors="surrogateescape").read()
for old, new in (("double operator * (double_eps &a,double &b)",
                  "double operator * (const double_eps &a,const double &b)"),
                 ("double operator * (double_eps &a,double_eps &b)",
                  "double operator * (const double_eps &a,const double_eps &b)")):
    assert src.count(old) == 1, "unexpected Subdomain source"
    src = src.replace(old, new)
sys.stdout.write(f'#line 1 "{path}"\n')
sys.stdout.write(src)
