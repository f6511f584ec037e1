#!/usr/bin/env bash
# Compile the reference's own general-XRCC C kernels from their sources in the read-only
# reference tree into oracle/_ref/ (git-ignored).  Test infrastructure only: the results
# check the NumPy restatement (oracle/xr_oracle.py) and time the reference CPU path.
#
#   general-XRCC/density_tensors.c  -> oracle/_ref/libref_density_tensors.so
#   general-XRCC/H_contractions.c   -> oracle/_ref/libref_H_contractions.so
#
# Flags follow the reference's own loader: qode.util.PyC.import_C(name, flags="-O2")
# (general-XRCC/build_H.py:20, general-XRCC/build_density_tensors.py:23-24).
# The reference tree is the first argument, else $XRH_REFERENCE_ROOT, else /root/reference.
# Without the sources (e.g. on a machine that has only this repository) it exits 0 and keeps
# any prebuilt oracle/_ref.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${XRH_REFERENCE_ROOT:-/root/reference}}"
SRC="$REF/general-XRCC"
OUT="$HERE/_ref"
if [ ! -f "$SRC/density_tensors.c" ]; then
    echo "reference sources not found under $SRC; keeping any prebuilt oracle/_ref" >&2
    exit 0
fi
mkdir -p "$OUT"
for k in density_tensors H_contractions; do
    gcc -O2 -shared -fPIC -std=gnu99 -I "$HERE/pyc_shim" "$SRC/$k.c" -o "$OUT/libref_$k.so.tmp"
    mv "$OUT/libref_$k.so.tmp" "$OUT/libref_$k.so"
done
echo "built: $(ls "$OUT")"
