function status = decaes_gpu(varargin)
%DECAES_GPU Run the decaes command line on the GPU library (decaes_gb300).
% The counterpart of the reference's api/decaes.m: the arguments are those of
% the decaes command line interface, given as strings, numbers or numeric
% arrays (each array element becomes one argument), for example
%
%   decaes_gpu('image.nii.gz', '--output', 'results', '--T2map', '--T2part', ...
%              '--TE', 7e-3, '--nT2', 40, '--T2Range', [7e-3, 2.0], ...
%              '--SPWin', [7e-3, 25e-3], '--MPWin', [25e-3, 200e-3], '--Reg', 'lcurve')
%
% MATLAB-side flags (not forwarded):
%   --python   Python interpreter, default 'python3'
%   --server   forward to a running warm daemon started with
%              'python -m decaes_gb300.daemon serve' (no per-call start-up)
%   --port     that daemon's port
%
% OUTPUT: status, the exit status of the call (see SYSTEM).

python = 'python3';
server = false;
port = '';
args = {};
i = 1;
while i <= numel(varargin)
    a = varargin{i};
    if ischar(a) && strcmp(a, '--python')
        python = varargin{i + 1}; i = i + 2; continue;
    elseif ischar(a) && strcmp(a, '--server')
        server = true; i = i + 1; continue;
    elseif ischar(a) && strcmp(a, '--port')
        port = num2str(varargin{i + 1}); i = i + 2; continue;
    end
    if ischar(a) || isstring(a)
        args{end + 1} = char(a); %#ok<AGROW>
    elseif isnumeric(a) || islogical(a)
        for v = double(a(:)')
            args{end + 1} = num2str(v, 17); %#ok<AGROW>
        end
    else
        error('decaes_gpu: arguments must be strings or numeric values');
    end
    i = i + 1;
end

here = fileparts(mfilename('fullpath'));
pkg = fileparts(here);  % the directory holding decaes_gb300/
quoted = cellfun(@(s) ['"', strrep(s, '"', '\"'), '"'], args, 'UniformOutput', false);
if server
    if isempty(port)
        cmd = sprintf('%s -m decaes_gb300.daemon run -- %s', python, strjoin(quoted, ' '));
    else
        cmd = sprintf('%s -m decaes_gb300.daemon run --port %s -- %s', python, port, strjoin(quoted, ' '));
    end
else
    cmd = sprintf('%s -m decaes_gb300 %s', python, strjoin(quoted, ' '));
end
old = getenv('PYTHONPATH');
if isempty(old)
    setenv('PYTHONPATH', pkg);
else
    setenv('PYTHONPATH', [pkg, pathsep, old]);
end
cleanup = onCleanup(@() setenv('PYTHONPATH', old));
st = system(cmd);
if nargout > 0
    status = st;
end
end
