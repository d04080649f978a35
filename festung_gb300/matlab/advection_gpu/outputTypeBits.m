% outputTypes ({'vtk'}, {'tec'} or both, core/visualizeDataLagr.m:104-112) as DGADV_OUT_* bits.
function bits = outputTypeBits(types)
if ~iscell(types)
  types = cellstr(types);
end % if
bits = 0;
for t = types(:)'
  if strcmp(t{1}, 'vtk')
    bits = bitor(bits, 1);
  elseif strcmp(t{1}, 'tec')
    bits = bitor(bits, 2);
  else
    error('Unknown file type: %s', t{1});
  end % if
end % for
end % function
